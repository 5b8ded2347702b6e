// dvm_noalloc.cu -- the collision integral for callers that cannot allocate device memory.
//
// Some hosts cannot call cudaMalloc: a solver embedded in a plugin whose host owns all
// device memory and forbids allocation behind its back, code that runs while a memory
// pool is pinned at a fixed budget, or a real-time loop that must not hit the driver's
// allocator. dvm_collide_noalloc serves them. It allocates nothing: the caller passes f and
// the cell properties in device memory, and every intermediate (velocity-grid tables,
// CDFs, bucket tables, sample plan, error word) lives in one file-scope device array of
// kNoAllocScratchBytes, which every GPU that loads this library holds until the process
// exits.
//
// Host code cannot use that array's name as a device address (it is a host-side
// stand-in), so the first call on each device looks the address up with
// cudaGetSymbolAddress, with that device current, and caches it; that first call should
// therefore come before any stream capture. The cached address belongs to the device's
// context as it was at that first call: do not use this entry point across a
// cudaDeviceReset (or anything else that tears the primary context down), after which the
// address would be stale. All calls share the array and it keeps the last call's
// contents: everything that must start from zero is cleared on every call, except the
// error word, which accumulates until a call that waits for its result reads and clears
// it. Calls that overlap on the GPU (other streams, other host threads) race on the array.
//
// Size: 16*(Nv+1) + 16112 bytes per cell (two 64-bit cumulative sums per node, the signs
// in their low bits, two 1000-entry bucket tables, the equilibrium cache, plan and chunk
// offsets) plus the grid tables (under 0.2 MB), in 32 MiB: 410 cells of 16^3, 141 of
// 24^3, 61 of 32^3, 32 of 40^3.
#include <cuda_runtime.h>

#include <cmath>
#include <cstring>
#include <mutex>

#include "../../include/dvm_gpu.h"
#include "dvm_internal.h"

namespace dvm {
namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB
constexpr int kMaxDevices = 64;

__device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
void* g_scratch_ptr[kMaxDevices] = {nullptr};
int g_collide_grid[kMaxDevices] = {0};

size_t align256(size_t v) { return (v + 255) & ~static_cast<size_t>(255); }

// Offsets of every buffer inside the scratch array. The error word comes first, at a fixed
// offset, so that calls of any size find the bits earlier calls left there.
struct Layout {
  size_t err, axes, tabs, gtab, trig, eq_cache, cum_eq, cum_dev, ref_eq, ref_dev, plan,
      chunk_off, total, end;
};

Layout layout(int nx, int ny, int nz, int ncells, int gtab_n) {
  const size_t nv1 = static_cast<size_t>(nx) * ny * nz + 1;
  const size_t C = static_cast<size_t>(ncells);
  const int nmax = nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz);
  Layout L;
  size_t o = 0;
  L.err = o; o = align256(o + sizeof(uint32_t));
  L.axes = o; o = align256(o + 2 * sizeof(double) * (nx + ny + nz));
  L.tabs = o; o = align256(o + 3 * sizeof(AxisEntry) * nmax);
  L.gtab = o; o = align256(o + sizeof(double2) * gtab_n);
  L.trig = o; o = align256(o + sizeof(double2) * kTrigN);
  L.eq_cache = o; o = align256(o + sizeof(double) * C * kEqCache);
  L.cum_eq = o; o = align256(o + sizeof(double) * C * nv1);
  L.cum_dev = o; o = align256(o + sizeof(double) * C * nv1);
  L.ref_eq = o; o = align256(o + sizeof(int2) * C * kNRef);
  L.ref_dev = o; o = align256(o + sizeof(int2) * C * kNRef);
  L.plan = o; o = align256(o + sizeof(CellPlan) * C);
  L.chunk_off = o; o = align256(o + sizeof(long long) * (3 * C + 1));
  L.total = o; o = align256(o + sizeof(long long));
  L.end = o;
  return L;
}

// The remap tables of build_collision_tables (dvm_api.cu), built on the device so that
// no host buffer is needed either.
__global__ void k_noalloc_tables(GridInfo g, AxisEntry* tab, int nmax, double2* gtab,
                                 int gtab_n, double h, double vhs, double2* trig,
                                 double two_pi) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  const double nan = __longlong_as_double(0x7FF8000000000000LL);
  if (t < 3 * nmax) {
    const int a = t / nmax, o = t - a * nmax;
    const double* v = (a == 0) ? g.x : (a == 1 ? g.y : g.z);
    const int n = (a == 0) ? g.nx : (a == 1 ? g.ny : g.nz);
    AxisEntry e;
    for (int q = 0; q < kTabW; ++q) { e.D[q] = nan; e.invD[q] = nan; e.T[q] = nan; }
    if (o < n) {
      for (int s = -kTabS; s <= kTabS; ++s) {
        if (s == 0 || o + s < 0 || o + s >= n) continue;
        const double d = v[o + s] - v[o];
        e.D[kTabS + s] = d;
        e.invD[kTabS + s] = 1.0 / d;
        if (o - s >= 0 && o - s < n) {
          const double ext = v[o - s] - v[o];
          e.T[kTabS + s] = ext * (ext - d);
        }
      }
    }
    tab[t] = e;
  }
  if (t < gtab_n) {
    const double gg = sqrt(static_cast<double>(t)) * h;
    gtab[t] = make_double2(gg, (vhs == 1.0) ? gg : pow(gg, vhs));
  }
  if (t < kTrigN) {
    const double ang = two_pi * (static_cast<double>(t) / kTrigN);
    trig[t] = make_double2(cos(ang), sin(ang));
  }
}

// Axes and node volumes arrive as a kernel parameter, so no host buffer is copied.
struct AxesParam {
  double v[6 * kMaxAxis];
};

__global__ void k_noalloc_axes(AxesParam ax, double* dst, int n) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x)
    dst[t] = ax.v[t];
}

// compute_beta (grid/velocity_grid.f90:486-540) into a fixed-size array.
void beta(const double* a, int n, double* b) {
  b[0] = a[1] - a[0];
  b[n - 1] = a[n - 1] - a[n - 2];
  for (int i = 1; i + 1 < n; ++i) b[i] = (a[i + 1] - a[i]) / 2.0 + (a[i] - a[i - 1]) / 2.0;
}

bool increasing(const double* a, int n) {
  for (int i = 1; i < n; ++i)
    if (!(a[i] > a[i - 1])) return false;
  return true;
}

int status_of(cudaError_t e) {
  if (e == cudaSuccess) return DVM_OK;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return DVM_ERR_NODEVICE;
  return DVM_ERR_CUDA;
}

}  // namespace
}  // namespace dvm

using namespace dvm;

extern "C" int dvm_collide_noalloc(const dvm_params* p, const dvm_vgrid* vg, double* f,
                                   const double* props, int ncells, uint64_t step,
                                   void* stream, int64_t* collisions) {
  if (!p || !vg || !f || !props || ncells < 1 || !vg->x || !vg->y || !vg->z)
    return DVM_ERR_PARAM;
  if (p->coll_method != DVM_COLL_VR && p->coll_method != DVM_COLL_FMC) return DVM_ERR_PARAM;
  if (p->precision != DVM_PREC_FP64) return DVM_ERR_PARAM;  // FP64 plain method only
  if (p->num_repl < 1 || p->num_repl > kMaxRepl || !(p->dt > 0.0) || !(p->Kn > 0.0) ||
      !(p->mass > 0.0) || !(p->alpha > 0.0) || p->samples_per_step < 0)
    return DVM_ERR_PARAM;
  if (p->samples_mode != DVM_SAMPLES_FIXED &&
      !(p->samples_mode == DVM_SAMPLES_FORMULA && p->coln_rms > 0.0))
    return DVM_ERR_PARAM;
  const int nx = vg->nx, ny = vg->ny, nz = vg->nz;
  if (nx < 3 || ny < 3 || nz < 3 || nx > kMaxAxis || ny > kMaxAxis || nz > kMaxAxis)
    return DVM_ERR_PARAM;
  if (!increasing(vg->x, nx) || !increasing(vg->y, ny) || !increasing(vg->z, nz))
    return DVM_ERR_PARAM;

  // cubic uniform grid -> table of g, g^(2-2 omega)
  bool cubic = (nx == ny && ny == nz);
  for (int i = 0; cubic && i < nx; ++i)
    if (vg->x[i] != vg->y[i] || vg->x[i] != vg->z[i]) cubic = false;
  const double h = (vg->x[nx - 1] - vg->x[0]) / static_cast<double>(nx - 1);
  for (int i = 0; cubic && i + 1 < nx; ++i)
    if (std::fabs((vg->x[i + 1] - vg->x[i]) - h) > 1e-12 * std::fabs(h)) cubic = false;
  const int gtab_n = cubic ? 3 * (nx - 1) * (nx - 1) + 1 : 0;
  const Layout L = layout(nx, ny, nz, ncells, gtab_n);
  if (L.end > kNoAllocScratchBytes) return DVM_ERR_TOO_LARGE;

  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return status_of(e);
  if (dev < 0 || dev >= kMaxDevices) return DVM_ERR_PARAM;
  int grid_blocks = 0;
  unsigned char* base = nullptr;
  {
    // once per device, with that device current: the scratch array's device address
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_scratch_ptr[dev]) {
      void* ptr = nullptr;
      e = cudaGetSymbolAddress(&ptr, g_noalloc_scratch);
      if (e != cudaSuccess) return status_of(e);
      g_scratch_ptr[dev] = ptr;
      int sms = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      g_collide_grid[dev] = sms;
    }
    base = static_cast<unsigned char*>(g_scratch_ptr[dev]);
    grid_blocks = g_collide_grid[dev];
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);

  // velocity grid: axes and node volumes into the scratch array
  AxesParam axp;
  double* hv = axp.v;
  double* hx = hv;
  double* hy = hx + nx;
  double* hz = hy + ny;
  std::memcpy(hx, vg->x, sizeof(double) * nx);
  std::memcpy(hy, vg->y, sizeof(double) * ny);
  std::memcpy(hz, vg->z, sizeof(double) * nz);
  double* hbx = hz + nz;
  double* hby = hbx + nx;
  double* hbz = hby + ny;
  beta(hx, nx, hbx);
  beta(hy, ny, hby);
  beta(hz, nz, hbz);
  double* d_axes = reinterpret_cast<double*>(base + L.axes);
  k_noalloc_axes<<<1, 256, 0, s>>>(axp, d_axes, 2 * (nx + ny + nz));
  if ((e = cudaGetLastError()) != cudaSuccess) return status_of(e);

  GridInfo g{};
  g.nx = nx; g.ny = ny; g.nz = nz; g.nv = nx * ny * nz;
  g.xv_min = hx[0]; g.yv_min = hy[0]; g.zv_min = hz[0];
  g.xv_factor = static_cast<double>(nx - 1) / (hx[nx - 1] - g.xv_min);
  g.yv_factor = static_cast<double>(ny - 1) / (hy[ny - 1] - g.yv_min);
  g.zv_factor = static_cast<double>(nz - 1) / (hz[nz - 1] - g.zv_min);
  double mn = hbx[0] * hby[0] * hbz[0];
  for (int k = 0; k < nz; ++k)
    for (int j = 0; j < ny; ++j)
      for (int i = 0; i < nx; ++i) {
        const double b3 = hbx[i] * hby[j] * hbz[k];
        if (b3 < mn) mn = b3;
      }
  g.beta3_min = mn;
  g.x = d_axes; g.y = g.x + nx; g.z = g.y + ny;
  g.bx = g.z + nz; g.by = g.bx + nx; g.bz = g.by + ny;

  const double pi = (p->pi_mode == DVM_PI_EXACT) ? kPiExact : kPiReference;
  const double vhs = 2.0 - 2.0 * (0.5 * (p->omega + p->omega));
  const int nmax = nx > ny ? (nx > nz ? nx : nz) : (ny > nz ? ny : nz);
  AxisEntry* d_tab = reinterpret_cast<AxisEntry*>(base + L.tabs);
  double2* d_gtab = reinterpret_cast<double2*>(base + L.gtab);
  double2* d_trig = reinterpret_cast<double2*>(base + L.trig);
  {
    int n = (3 * nmax > gtab_n) ? 3 * nmax : gtab_n;
    n = n > kTrigN ? n : kTrigN;
    k_noalloc_tables<<<(n + 255) / 256, 256, 0, s>>>(g, d_tab, nmax, d_gtab, gtab_n, h, vhs,
                                                     d_trig, 2.0 * pi);
    if ((e = cudaGetLastError()) != cudaSuccess) return status_of(e);
  }
  // state that must start from zero: the equilibrium cache, so every call builds the
  // Maxwellian afresh, as a new context's first call does. The error word is not cleared
  // here: it collects the bits of every call since the last call that read it (one with
  // `collisions` set), so an error of a call that did not wait is reported by the next
  // call that does.
  uint32_t* d_err = reinterpret_cast<uint32_t*>(base + L.err);
  double* d_eq_cache = reinterpret_cast<double*>(base + L.eq_cache);
  if ((e = cudaMemsetAsync(d_eq_cache, 0, sizeof(double) * kEqCache * ncells, s)) != cudaSuccess)
    return status_of(e);

  CollParams cp;
  cp.method = p->coll_method;
  cp.samples_mode = p->samples_mode;
  cp.samples_per_step = p->samples_per_step;
  cp.num_repl = p->num_repl;
  cp.mass = p->mass; cp.omega = p->omega; cp.alpha = p->alpha; cp.sigma = p->sigma;
  cp.dt = p->dt; cp.Kn = p->Kn; cp.coln_rms = p->coln_rms;
  cp.cdf_tolerance = p->cdf_tolerance;
  cp.pi = pi;
  cp.seed = p->seed;
  {
    const double b3a = g.beta3_min * std::pow(p->mass, 3.0 / 2.0);
    cp.b3 = 0.5 * (b3a + b3a);
  }

  CdfArgs ca{};
  ca.g = g; ca.cp = cp; ca.ncells = ncells; ca.f = f; ca.props = props;
  ca.eq_cache = d_eq_cache;
  ca.cum_eq = reinterpret_cast<long long*>(base + L.cum_eq);
  ca.cum_dev = reinterpret_cast<long long*>(base + L.cum_dev);
  ca.ref_eq = reinterpret_cast<int2*>(base + L.ref_eq);
  ca.ref_dev = reinterpret_cast<int2*>(base + L.ref_dev);
  ca.plan = reinterpret_cast<CellPlan*>(base + L.plan);
  ca.err = d_err;
  if ((e = launch_cdf(ca, s)) != cudaSuccess) return status_of(e);
  long long* d_chunk = reinterpret_cast<long long*>(base + L.chunk_off);
  long long* d_total = reinterpret_cast<long long*>(base + L.total);
  // (the collide launch below has up to 4 CTAs per SM)
  if ((e = launch_plan(ncells, ca.plan, d_chunk, d_total,
                       static_cast<long long>(grid_blocks) * 4 * (kCollideChunk / 32), s)) !=
      cudaSuccess)
    return status_of(e);

  CollideArgs a{};
  a.g = g; a.cp = cp; a.ncells = ncells; a.step = static_cast<uint32_t>(step);
  a.t.axis = d_tab; a.t.nmax = nmax;
  a.t.gtab = cubic ? d_gtab : nullptr;
  a.t.gtab_n = gtab_n;
  a.t.gtab_smem = cubic ? gtab_staged(gtab_n) : 0;
  a.t.phi_scale = 2.0 * pi / kPiExact;
  a.t.trig = d_trig;
  a.t.two_pi = 2.0 * pi;
  a.f = f; a.cum_eq = ca.cum_eq; a.cum_dev = ca.cum_dev;
  a.ref_eq = ca.ref_eq; a.ref_dev = ca.ref_dev; a.plan = ca.plan; a.chunk_off = d_chunk;
  a.err = d_err;
  if ((e = launch_collide(a, grid_blocks * collide_blocks_per_sm(collide_smem_bytes(g, a.t)), s)) !=
      cudaSuccess)
    return status_of(e);

  if (collisions) {
    long long total = 0;
    uint32_t word = 0;
    if ((e = cudaMemcpyAsync(&total, d_total, sizeof(total), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaMemcpyAsync(&word, d_err, sizeof(word), cudaMemcpyDeviceToHost, s)) !=
            cudaSuccess ||
        (e = cudaMemsetAsync(d_err, 0, sizeof(uint32_t), s)) != cudaSuccess ||
        (e = cudaStreamSynchronize(s)) != cudaSuccess)
      return status_of(e);
    *collisions = total;
    if (word) return DVM_ERR_NUMERIC;
  }
  return DVM_OK;
}
