// dvm_api.cu -- the C ABI (include/dvm_gpu.h): context, device buffers, launch sequence.
//
// The context owns every device buffer (f, f_conv, properties, CDFs, ghosts), like
// phi / delta_phi / properties in initialize_solver (solver/dvm_solver.f90:55-64). Host
// arrays passed in are only borrowed for the duration of the call.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <vector>

#include "../../include/dvm_gpu.h"
#include "dvm_internal.h"

using namespace dvm;

struct dvm_ctx {
  dvm_params p{};
  GridInfo g{};
  int ncells = 0;
  double pi = kPiReference;
  int device = 0;
  int num_sms = 0;
  cudaStream_t stream = nullptr;
  // host copies of grid metadata
  std::vector<double> hx, hy, hz, hbx, hby, hbz;
  // device buffers
  double* d_axes = nullptr;   // x, y, z, bx, by, bz
  float2* d_speed = nullptr;  // |xi| per node as a hi + lo float pair
  double* d_f = nullptr;
  double* d_fconv = nullptr;
  double* d_props = nullptr;
  double* d_eq_cache = nullptr;
  long long* d_cum_eq = nullptr;   // fixed-point CDFs
  long long* d_cum_dev = nullptr;
  int2* d_ref_eq = nullptr;
  int2* d_ref_dev = nullptr;
  CellPlan* d_plan = nullptr;
  long long* d_chunk_off = nullptr;
  long long* d_total_samples = nullptr;
  double* d_ghost = nullptr;
  float2* d_cfl = nullptr;      // 2-D upwind |CFL| per axis node as hi + lo pairs
  uint32_t* d_err = nullptr;
  double* d_flush = nullptr;
  size_t flush_n = 0;
  AxisEntry* d_axis_tab = nullptr;
  double2* d_gtab = nullptr;
  double2* d_trig = nullptr;
  CollTables tabs{};
  // precision form: FP32 increment and FP32 tables
  float* d_df = nullptr;
  AxisEntryF* d_axis_tab_f = nullptr;
  float2* d_gtab_f = nullptr;
  float2* d_trig_f = nullptr;
  CollTablesF tabs_f{};
  int collide_f32_grid = 0;
  int wall_base[4] = {-1, -1, -1, -1};
  int wall_entries = 0;
  int collide_grid = 0;
  bool own_stream = true;
  bool async_alloc = false;                    // stream-ordered allocation on `stream`
  size_t device_bytes = 0;                     // bytes this context allocated
  const uint32_t* step_dev = nullptr;          // set when a batch owns the step counter
  unsigned long long* d_residual = nullptr;    // convergence residual of the last moments
  // instrumentation
  bool profile = false;
  std::vector<cudaEvent_t> ev_pool;
  struct Rec { int kid; cudaEvent_t a, b; };
  std::vector<Rec> recs;
  double prof_ms[DVM_K_COUNT] = {0};
  int64_t prof_n[DVM_K_COUNT] = {0};
  int64_t launches = 0;
};

namespace {

const char* kKernelNames[DVM_K_COUNT] = {"cdf_build", "collide_plan", "collide", "wall_flux",
                                         "wall_ghost", "convect", "bc_1d", "moments",
                                         "project"};

int cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return DVM_OK;
  if (e == cudaErrorMemoryAllocation) return DVM_ERR_OOM;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return DVM_ERR_NODEVICE;
  return DVM_ERR_CUDA;
}

cudaEvent_t take_event(dvm_ctx* c) {
  if (!c->ev_pool.empty()) {
    cudaEvent_t e = c->ev_pool.back();
    c->ev_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

// Runs one launch wrapper, counting it and, when profiling, bracketing it with events.
template <typename F>
int launch(dvm_ctx* c, int kid, F&& fn) {
  cudaEvent_t a = nullptr, b = nullptr;
  if (c->profile) {
    a = take_event(c);
    b = take_event(c);
    cudaEventRecord(a, c->stream);
  }
  cudaError_t e = fn();
  if (c->profile) {
    cudaEventRecord(b, c->stream);
    c->recs.push_back({kid, a, b});
  }
  c->launches++;
  return cuda_status(e);
}

void harvest(dvm_ctx* c) {
  if (c->recs.empty()) return;
  cudaStreamSynchronize(c->stream);
  for (auto& r : c->recs) {
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, r.a, r.b) == cudaSuccess) c->prof_ms[r.kid] += ms;
    c->prof_n[r.kid]++;
    c->ev_pool.push_back(r.a);
    c->ev_pool.push_back(r.b);
  }
  c->recs.clear();
}

// compute_beta, grid/velocity_grid.f90:486-540
void node_volumes(const std::vector<double>& a, std::vector<double>& b) {
  const size_t n = a.size();
  b.resize(n);
  b[0] = a[1] - a[0];
  b[n - 1] = a[n - 1] - a[n - 2];
  for (size_t i = 1; i + 1 < n; ++i) b[i] = (a[i + 1] - a[i]) / 2.0 + (a[i] - a[i - 1]) / 2.0;
}

// find_zero_point, grid/velocity_grid.f90:653-689
void zero_point(const std::vector<double>& a, int& zero, int& pos, int& neg) {
  const int n = static_cast<int>(a.size());
  if (a[0] > 0.0) { zero = -1; pos = 0; neg = -1; return; }
  for (int i = 1; i < n; ++i) {
    if (a[i] > 0.0) {
      zero = i - 1; pos = i; neg = i - 1;
      if (a[i - 1] > -kDoubleTol) neg = i - 2;
      return;
    }
  }
  zero = n; pos = n; neg = n - 1;
}

template <typename T>
int dalloc(T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return DVM_OK;
  return cuda_status(cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T)));
}

// Context allocation: stream-ordered for server-owned contexts, so that creating or freeing
// one never waits for the work of others.
template <typename T>
int dalloc(dvm_ctx* c, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) return DVM_OK;
  const size_t bytes = count * sizeof(T);
  cudaError_t e = c->async_alloc
                      ? cudaMallocAsync(reinterpret_cast<void**>(p), bytes, c->stream)
                      : cudaMalloc(reinterpret_cast<void**>(p), bytes);
  if (e == cudaSuccess) c->device_bytes += bytes;
  return cuda_status(e);
}

int h2d(dvm_ctx* c, void* dst, const void* src, size_t bytes) {
  return cuda_status(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, c->stream));
}

void release(dvm_ctx* c) {
  if (!c) return;
  harvest(c);
  for (auto e : c->ev_pool) cudaEventDestroy(e);
  void* bufs[] = {c->d_axes, c->d_speed, c->d_f, c->d_fconv, c->d_props, c->d_eq_cache,
                  c->d_cum_eq, c->d_cum_dev, c->d_ref_eq, c->d_ref_dev, c->d_plan,
                  c->d_chunk_off, c->d_total_samples, c->d_ghost, c->d_err, c->d_flush,
                  c->d_axis_tab, c->d_gtab, c->d_trig, c->d_df, c->d_axis_tab_f,
                  c->d_gtab_f, c->d_trig_f, c->d_residual, c->d_cfl};
  for (void* b : bufs)
    if (b) {
      if (c->async_alloc) cudaFreeAsync(b, c->stream);
      else cudaFree(b);
    }
  if (c->stream && c->own_stream) cudaStreamDestroy(c->stream);
  delete c;
}

bool increasing(const double* a, int n) {
  for (int i = 1; i < n; ++i)
    if (!(a[i] > a[i - 1])) return false;
  return true;
}

int validate(const dvm_params* p, const dvm_vgrid* vg) {
  if (!p || !vg || !vg->x || !vg->y || !vg->z) return DVM_ERR_PARAM;
  if (vg->nx < 3 || vg->ny < 3 || vg->nz < 3) return DVM_ERR_PARAM;
  if (vg->nx > kMaxAxis || vg->ny > kMaxAxis || vg->nz > kMaxAxis) return DVM_ERR_PARAM;
  if (!increasing(vg->x, vg->nx) || !increasing(vg->y, vg->ny) || !increasing(vg->z, vg->nz))
    return DVM_ERR_PARAM;
  if (p->nx_space < 1 || p->ny_space < 1) return DVM_ERR_PARAM;
  if (p->coll_method != DVM_COLL_NONE && p->coll_method != DVM_COLL_FMC &&
      p->coll_method != DVM_COLL_VR)
    return DVM_ERR_PARAM;
  if (p->conv_method != DVM_CONV_NONE && p->conv_method != DVM_CONV_UPWIND1) return DVM_ERR_PARAM;
  if (p->num_repl < 1 || p->num_repl > kMaxRepl) return DVM_ERR_PARAM;
  if (p->samples_mode != DVM_SAMPLES_FORMULA && p->samples_mode != DVM_SAMPLES_FIXED)
    return DVM_ERR_PARAM;
  if (p->samples_per_step < 0) return DVM_ERR_PARAM;
  if (p->precision != DVM_PREC_FP64 && p->precision != DVM_PREC_FP32) return DVM_ERR_PARAM;
  if (!(p->dt > 0.0) || !(p->Kn > 0.0) || !(p->mass > 0.0)) return DVM_ERR_PARAM;
  if (p->coll_method != DVM_COLL_NONE && !(p->alpha > 0.0)) return DVM_ERR_PARAM;
  if (p->samples_mode == DVM_SAMPLES_FORMULA && p->coll_method != DVM_COLL_NONE &&
      !(p->coln_rms > 0.0))
    return DVM_ERR_PARAM;
  if (p->conv_method == DVM_CONV_UPWIND1) {
    if (p->geometry == DVM_GEOM_2D) {
      if (p->nx_space < 2 || p->ny_space < 2 || !(p->dx > 0.0) || !(p->dy > 0.0))
        return DVM_ERR_PARAM;
    } else if (p->geometry == DVM_GEOM_1D) {
      // ny_space > 1: that many independent rows of nx_space cells (a batch of 1-D
      // instances), each with both end conditions
      if (p->nx_space < 3 || p->ny_space < 1 || !(p->dx > 0.0)) return DVM_ERR_PARAM;
      for (int e = 0; e < 2; ++e)
        if (p->bc[e] < DVM_BC1D_SPECULAR || p->bc[e] > DVM_BC1D_ZEROGRAD) return DVM_ERR_PARAM;
    } else {
      return DVM_ERR_PARAM;  // 0-D has no convection
    }
  }
  if (p->geometry < DVM_GEOM_0D || p->geometry > DVM_GEOM_2D) return DVM_ERR_PARAM;
  if (p->geometry == DVM_GEOM_0D && (p->nx_space != 1 || p->ny_space != 1)) {
    // independent homogeneous cells are allowed (a batch of 0-D instances on one grid)
    if (p->conv_method != DVM_CONV_NONE) return DVM_ERR_PARAM;
  }
  return DVM_OK;
}

// Remap tables per axis and, on a cubic uniform grid, the table of g and g^(2-2 omega)
// indexed by di^2 + dj^2 + dk^2 (see CollTables).
int build_collision_tables(dvm_ctx* c) {
  const GridInfo& g = c->g;
  const std::vector<double>* ax[3] = {&c->hx, &c->hy, &c->hz};
  const int nmax = std::max(g.nx, std::max(g.ny, g.nz));
  std::vector<AxisEntry> tab(3 * static_cast<size_t>(nmax));
  const double nan = std::nan("");
  for (int a = 0; a < 3; ++a) {
    const std::vector<double>& v = *ax[a];
    const int n = static_cast<int>(v.size());
    for (int o = 0; o < nmax; ++o) {
      AxisEntry& e = tab[static_cast<size_t>(a) * nmax + o];
      for (int q = 0; q < kTabW; ++q) { e.D[q] = nan; e.invD[q] = nan; e.T[q] = nan; }
      if (o >= n) continue;
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
  }
  int st = dalloc(c, &c->d_axis_tab, tab.size());
  if (st) return st;
  h2d(c, c->d_axis_tab, tab.data(), tab.size() * sizeof(AxisEntry));
  c->tabs.axis = c->d_axis_tab;
  c->tabs.nmax = nmax;
  c->tabs.phi_scale = 2.0 * c->pi / kPiExact;
  c->tabs.two_pi = 2.0 * c->pi;
  {
    std::vector<double2> tr(kTrigN);
    for (int k = 0; k < kTrigN; ++k) {
      const double ang = 2.0 * c->pi * (static_cast<double>(k) / kTrigN);
      tr[k].x = std::cos(ang);
      tr[k].y = std::sin(ang);
    }
    if ((st = dalloc(c, &c->d_trig, tr.size()))) return st;
    h2d(c, c->d_trig, tr.data(), tr.size() * sizeof(double2));
    c->tabs.trig = c->d_trig;
  }
  // cubic uniform grid: the same uniform axis three times
  bool cubic = (g.nx == g.ny && g.ny == g.nz && c->hx == c->hy && c->hy == c->hz);
  const int n = g.nx;
  const double h = (c->hx[n - 1] - c->hx[0]) / static_cast<double>(n - 1);
  for (int i = 0; cubic && i + 1 < n; ++i)
    if (std::fabs((c->hx[i + 1] - c->hx[i]) - h) > 1e-12 * std::fabs(h)) cubic = false;
  c->tabs.gtab = nullptr;
  c->tabs.gtab_n = 0;
  c->tabs.gtab_smem = 0;
  if (cubic) {
    const int ns = 3 * (n - 1) * (n - 1) + 1;
    const double vhs = 2.0 - 2.0 * (0.5 * (c->p.omega + c->p.omega));
    std::vector<double2> gt(ns);
    for (int s2 = 0; s2 < ns; ++s2) {
      const double gg = std::sqrt(static_cast<double>(s2)) * h;
      gt[s2].x = gg;
      gt[s2].y = (vhs == 1.0) ? gg : std::pow(gg, vhs);
    }
    if ((st = dalloc(c, &c->d_gtab, gt.size()))) return st;
    h2d(c, c->d_gtab, gt.data(), gt.size() * sizeof(double2));
    c->tabs.gtab = c->d_gtab;
    c->tabs.gtab_n = ns;
    c->tabs.gtab_smem = gtab_staged(ns);
  }
  if (c->p.precision == DVM_PREC_FP32) {
    // FP32 copies of the same tables for k_collide_f32
    std::vector<AxisEntryF> tf(tab.size());
    for (size_t e = 0; e < tab.size(); ++e)
      for (int q = 0; q < kTabW; ++q) {
        tf[e].D[q] = static_cast<float>(tab[e].D[q]);
        tf[e].invD[q] = static_cast<float>(tab[e].invD[q]);
        tf[e].T[q] = static_cast<float>(tab[e].T[q]);
      }
    if ((st = dalloc(c, &c->d_axis_tab_f, tf.size()))) return st;
    h2d(c, c->d_axis_tab_f, tf.data(), tf.size() * sizeof(AxisEntryF));
    std::vector<float2> trf(kTrigN);
    for (int k = 0; k < kTrigN; ++k) {
      const double ang = 2.0 * c->pi * (static_cast<double>(k) / kTrigN);
      trf[k] = make_float2(static_cast<float>(std::cos(ang)), static_cast<float>(std::sin(ang)));
    }
    if ((st = dalloc(c, &c->d_trig_f, trf.size()))) return st;
    h2d(c, c->d_trig_f, trf.data(), trf.size() * sizeof(float2));
    c->tabs_f.axis = c->d_axis_tab_f;
    c->tabs_f.trig = c->d_trig_f;
    c->tabs_f.two_pi = static_cast<float>(2.0 * c->pi);
    c->tabs_f.gtab = nullptr;
    c->tabs_f.gtab_smem = 0;
    if (c->tabs.gtab) {
      const int ns = c->tabs.gtab_n;
      const double vhs = 2.0 - 2.0 * (0.5 * (c->p.omega + c->p.omega));
      std::vector<float2> gf(ns);
      for (int s2 = 0; s2 < ns; ++s2) {
        const double gg = std::sqrt(static_cast<double>(s2)) * h;
        gf[s2] = make_float2(static_cast<float>(gg),
                             static_cast<float>((vhs == 1.0) ? gg : std::pow(gg, vhs)));
      }
      if ((st = dalloc(c, &c->d_gtab_f, gf.size()))) return st;
      h2d(c, c->d_gtab_f, gf.data(), gf.size() * sizeof(float2));
      c->tabs_f.gtab = c->d_gtab_f;
      c->tabs_f.gtab_smem = (static_cast<size_t>(ns) * sizeof(float2) <= 48 * 1024) ? 1 : 0;
    }
    const size_t n = static_cast<size_t>(c->ncells) * c->g.nv;
    if ((st = dalloc(c, &c->d_df, n))) return st;
    cudaMemsetAsync(c->d_df, 0, n * sizeof(float), c->stream);
    const bool fast = c->p.num_repl == 1 && c->tabs.gtab != nullptr &&
                      !(std::fabs(1.0 / (0.5 * (c->p.alpha + c->p.alpha)) - 1.0) > kDoubleTol);
    c->collide_f32_grid = c->num_sms * collide_f32_blocks_per_sm(c->g, c->tabs, fast);
  }
  // the host tables above are staged before they go out of scope
  return cuda_status(cudaStreamSynchronize(c->stream));
}

CollParams coll_params(const dvm_ctx* c) {
  CollParams cp;
  cp.method = c->p.coll_method;
  cp.samples_mode = c->p.samples_mode;
  cp.samples_per_step = c->p.samples_per_step;
  cp.num_repl = c->p.num_repl;
  cp.mass = c->p.mass;
  cp.omega = c->p.omega;
  cp.alpha = c->p.alpha;
  cp.sigma = c->p.sigma;
  cp.dt = c->p.dt;
  cp.Kn = c->p.Kn;
  cp.coln_rms = c->p.coln_rms;
  cp.cdf_tolerance = c->p.cdf_tolerance;
  cp.pi = c->pi;
  cp.seed = c->p.seed;
  // compute_num_coll_pairs (collision_utilities.f90:106-140): beta3_min * m^(3/2), averaged
  // over the (like-species) pair
  const double b3a = c->g.beta3_min * std::pow(c->p.mass, 3.0 / 2.0);
  cp.b3 = 0.5 * (b3a + b3a);
  return cp;
}

}  // namespace

int create_context(const dvm_params* params, const dvm_vgrid* vg, cudaStream_t stream,
                   bool async_alloc, dvm_ctx** out);

extern "C" {

int dvm_abi_version(void) { return DVM_ABI_VERSION; }

const char* dvm_strerror(int status) {
  switch (status) {
    case DVM_OK: return "ok";
    case DVM_ERR_PARAM: return "invalid parameter";
    case DVM_ERR_OOM: return "device memory allocation failed";
    case DVM_ERR_CUDA: return "CUDA error";
    case DVM_ERR_NUMERIC: return "device error word set";
    case DVM_ERR_TIMEOUT: return "device wait timed out";
    case DVM_ERR_NODEVICE: return "no CUDA device";
    case DVM_ERR_TOO_LARGE: return "problem exceeds the 32 MiB no-allocation scratch array";
    case DVM_ERR_IO: return "an output file could not be opened or written";
    default: return "unknown status";
  }
}

const char* dvm_kernel_name(int kid) {
  return (kid >= 0 && kid < DVM_K_COUNT) ? kKernelNames[kid] : "unknown";
}

int dvm_create(const dvm_params* params, const dvm_vgrid* vg, dvm_ctx** out) {
  return create_context(params, vg, nullptr, false, out);
}

}  // extern "C"

// A context on the caller's stream (stream != null: batches share one stream).
int create_context(const dvm_params* params, const dvm_vgrid* vg, cudaStream_t stream,
                   bool async_alloc, dvm_ctx** out) {
  if (!out) return DVM_ERR_PARAM;
  *out = nullptr;
  int st = validate(params, vg);
  if (st) return st;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev < 1) return DVM_ERR_NODEVICE;
  dvm_ctx* c = new (std::nothrow) dvm_ctx();
  if (!c) return DVM_ERR_OOM;
  c->p = *params;
  c->pi = (params->pi_mode == DVM_PI_EXACT) ? kPiExact : kPiReference;
  c->ncells = params->nx_space * params->ny_space;
  cudaGetDevice(&c->device);
  cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, c->device);
  c->async_alloc = async_alloc;
  if (stream) {
    c->stream = stream;
    c->own_stream = false;
  } else if ((st = cuda_status(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking)))) {
    release(c);
    return st;
  }
  c->hx.assign(vg->x, vg->x + vg->nx);
  c->hy.assign(vg->y, vg->y + vg->ny);
  c->hz.assign(vg->z, vg->z + vg->nz);
  node_volumes(c->hx, c->hbx);
  node_volumes(c->hy, c->hby);
  node_volumes(c->hz, c->hbz);
  GridInfo& g = c->g;
  g.nx = vg->nx; g.ny = vg->ny; g.nz = vg->nz;
  g.nv = g.nx * g.ny * g.nz;
  g.xv_min = c->hx[0]; g.yv_min = c->hy[0]; g.zv_min = c->hz[0];
  // create_velocity_grid, grid/velocity_grid.f90:293-313
  g.xv_factor = static_cast<double>(g.nx - 1) / (c->hx[g.nx - 1] - g.xv_min);
  g.yv_factor = static_cast<double>(g.ny - 1) / (c->hy[g.ny - 1] - g.yv_min);
  g.zv_factor = static_cast<double>(g.nz - 1) / (c->hz[g.nz - 1] - g.zv_min);
  zero_point(c->hx, g.i_zero, g.i_pos, g.i_neg);
  zero_point(c->hy, g.j_zero, g.j_pos, g.j_neg);
  // set_boundary_nodes :676-684 (SAVEd flags; one grid per context)
  g.i_zero_flag = (g.i_zero != 0 && g.i_zero != g.i_neg && g.i_zero != g.i_pos && g.i_zero != g.nx - 1);
  g.j_zero_flag = (g.j_zero != 0 && g.j_zero != g.j_neg && g.j_zero != g.j_pos && g.j_zero != g.ny - 1);
  // find_min_max_beta3, grid/velocity_grid.f90:542-597
  double mn = c->hbx[0] * c->hby[0] * c->hbz[0];
  for (int k = 0; k < g.nz; ++k)
    for (int j = 0; j < g.ny; ++j)
      for (int i = 0; i < g.nx; ++i) mn = std::min(mn, c->hbx[i] * c->hby[j] * c->hbz[k]);
  g.beta3_min = mn;

  const size_t C = c->ncells, nv = g.nv;
  const size_t naxes = 2 * (g.nx + g.ny + g.nz);
  if ((st = dalloc(c, &c->d_axes, naxes)) || (st = dalloc(c, &c->d_f, C * nv)) ||
      (st = dalloc(c, &c->d_fconv, C * nv)) || (st = dalloc(c, &c->d_props, C * DVM_NPROP)) ||
      (st = dalloc(c, &c->d_err, 1))) {
    release(c);
    return st;
  }
  if (params->coll_method != DVM_COLL_NONE) {
    if ((st = dalloc(c, &c->d_eq_cache, C * kEqCache)) ||
        (st = dalloc(c, &c->d_cum_eq, C * (nv + 1))) || (st = dalloc(c, &c->d_cum_dev, C * (nv + 1))) ||
        (st = dalloc(c, &c->d_ref_eq, C * kNRef)) ||
        (st = dalloc(c, &c->d_ref_dev, C * kNRef)) || (st = dalloc(c, &c->d_plan, C)) ||
        (st = dalloc(c, &c->d_chunk_off, 3 * C + 1)) || (st = dalloc(c, &c->d_total_samples, 2))) {
      release(c);
      return st;
    }
  }
  // axes on the device: x, y, z, bx, by, bz
  std::vector<double> axes;
  axes.insert(axes.end(), c->hx.begin(), c->hx.end());
  axes.insert(axes.end(), c->hy.begin(), c->hy.end());
  axes.insert(axes.end(), c->hz.begin(), c->hz.end());
  axes.insert(axes.end(), c->hbx.begin(), c->hbx.end());
  axes.insert(axes.end(), c->hby.begin(), c->hby.end());
  axes.insert(axes.end(), c->hbz.begin(), c->hbz.end());
  h2d(c, c->d_axes, axes.data(), naxes * sizeof(double));
  g.x = c->d_axes;
  g.y = g.x + g.nx;
  g.z = g.y + g.ny;
  g.bx = g.z + g.nz;
  g.by = g.bx + g.nx;
  g.bz = g.by + g.ny;
  {
    std::vector<double> sp(nv);
    size_t l = 0;
    for (int k = 0; k < g.nz; ++k)
      for (int j = 0; j < g.ny; ++j)
        for (int i = 0; i < g.nx; ++i, ++l)
          sp[l] = std::sqrt(c->hx[i] * c->hx[i] + c->hy[j] * c->hy[j] + c->hz[k] * c->hz[k]);
    if ((st = dalloc(c, &c->d_speed, nv))) {
      release(c);
      return st;
    }
    std::vector<float2> sp2(nv);
    for (size_t l = 0; l < nv; ++l) {
      const float h = static_cast<float>(sp[l]);
      sp2[l] = make_float2(h, static_cast<float>(sp[l] - static_cast<double>(h)));
    }
    h2d(c, c->d_speed, sp2.data(), nv * sizeof(float2));
    g.speed = c->d_speed;
    cudaStreamSynchronize(c->stream);
  }
  cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream);
  cudaMemsetAsync(c->d_f, 0, C * nv * sizeof(double), c->stream);
  cudaMemsetAsync(c->d_props, 0, C * DVM_NPROP * sizeof(double), c->stream);
  if (c->d_eq_cache) cudaMemsetAsync(c->d_eq_cache, 0, C * kEqCache * sizeof(double), c->stream);
  // 2-D wall ghost entries: left/right walls (if walls), bottom and top (always walls)
  if (params->geometry == DVM_GEOM_2D && params->conv_method == DVM_CONV_UPWIND1) {
    int n = 0;
    const int NXS = params->nx_space, NYS = params->ny_space;
    if (params->bc[DVM_WALL_LEFT] == DVM_BC2D_WALL) { c->wall_base[0] = n; n += NYS; }
    if (params->bc[DVM_WALL_RIGHT] == DVM_BC2D_WALL) { c->wall_base[1] = n; n += NYS; }
    c->wall_base[2] = n; n += NXS;
    c->wall_base[3] = n; n += NXS;
    c->wall_entries = n;
    if ((st = dalloc(c, &c->d_ghost, static_cast<size_t>(n) * nv))) {
      release(c);
      return st;
    }
    // |dt/dx x_i|, |dt/dy y_j| split into float pairs for the convection kernel
    std::vector<float2> cfl(g.nx + g.ny);
    for (int i = 0; i < g.nx + g.ny; ++i) {
      const double v = (i < g.nx) ? std::fabs(params->dt / params->dx * c->hx[i])
                                  : std::fabs(params->dt / params->dy * c->hy[i - g.nx]);
      const float h = static_cast<float>(v);
      cfl[i] = make_float2(h, static_cast<float>(v - static_cast<double>(h)));
    }
    if ((st = dalloc(c, &c->d_cfl, cfl.size()))) {
      release(c);
      return st;
    }
    h2d(c, c->d_cfl, cfl.data(), cfl.size() * sizeof(float2));
    cudaStreamSynchronize(c->stream);
  }
  if (params->coll_method != DVM_COLL_NONE) {
    if ((st = build_collision_tables(c))) {
      release(c);
      return st;
    }
    const int bps = collide_blocks_per_sm(collide_smem_bytes(g, c->tabs));
    c->collide_grid = c->num_sms * bps;
  }
  if ((st = dalloc(c, &c->d_residual, 1))) {
    release(c);
    return st;
  }
  cudaMemsetAsync(c->d_residual, 0, sizeof(unsigned long long), c->stream);
  // host staging vectors above outlive this synchronisation
  if ((st = cuda_status(cudaStreamSynchronize(c->stream)))) {
    release(c);
    return st;
  }
  *out = c;
  return DVM_OK;
}

extern "C" {

int dvm_destroy(dvm_ctx* c) {
  if (!c) return DVM_ERR_PARAM;
  release(c);
  return DVM_OK;
}

int dvm_num_velocity_points(const dvm_ctx* c) { return c ? c->g.nv : -1; }
int dvm_num_cells(const dvm_ctx* c) { return c ? c->ncells : -1; }

int dvm_upload_f(dvm_ctx* c, const double* f) {
  if (!c || !f) return DVM_ERR_PARAM;
  const size_t bytes = static_cast<size_t>(c->ncells) * c->g.nv * sizeof(double);
  int st = cuda_status(cudaMemcpyAsync(c->d_f, f, bytes, cudaMemcpyHostToDevice, c->stream));
  if (st) return st;
  // initialize_solver computes the properties of the initial state
  st = dvm_calculate_physical_properties(c);
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(c->stream));
}

int dvm_download_f(dvm_ctx* c, double* f) {
  if (!c || !f) return DVM_ERR_PARAM;
  const size_t bytes = static_cast<size_t>(c->ncells) * c->g.nv * sizeof(double);
  int st = cuda_status(cudaMemcpyAsync(f, c->d_f, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(c->stream));
}

int dvm_calculate_physical_properties(dvm_ctx* c) {
  if (!c) return DVM_ERR_PARAM;
  MomentArgs a{c->g, c->ncells, c->p.mass, c->d_f, c->d_props, c->d_err, c->d_residual,
               nullptr};
  int st = cuda_status(cudaMemsetAsync(c->d_residual, 0, sizeof(unsigned long long), c->stream));
  if (st) return st;
  return launch(c, DVM_K_MOMENTS, [&] { return launch_moments(a, c->stream); });
}

int dvm_get_properties(dvm_ctx* c, double* props) {
  if (!c || !props) return DVM_ERR_PARAM;
  const size_t bytes = static_cast<size_t>(c->ncells) * DVM_NPROP * sizeof(double);
  int st = cuda_status(cudaMemcpyAsync(props, c->d_props, bytes, cudaMemcpyDeviceToHost, c->stream));
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(c->stream));
}

int dvm_set_properties(dvm_ctx* c, const double* props) {
  if (!c || !props) return DVM_ERR_PARAM;
  const size_t bytes = static_cast<size_t>(c->ncells) * DVM_NPROP * sizeof(double);
  int st = cuda_status(cudaMemcpyAsync(c->d_props, props, bytes, cudaMemcpyHostToDevice, c->stream));
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(c->stream));
}

int dvm_compute_collision_integral(dvm_ctx* c, uint64_t step, const dvm_pairlist* pairs) {
  if (!c) return DVM_ERR_PARAM;
  if (c->p.coll_method == DVM_COLL_NONE) return DVM_OK;
  PairDev pd{};
  std::vector<void*> tmp;
  int st = DVM_OK;
  if (pairs) {
    pd.active = 1;
    const int NR = c->p.num_repl;
    const int nsub = (c->p.coll_method == DVM_COLL_VR) ? 3 : 1;
    auto up = [&](const void* src, size_t bytes) -> void* {
      if (!src || bytes == 0) return nullptr;
      void* d = nullptr;
      if (cudaMalloc(&d, bytes) != cudaSuccess) { st = DVM_ERR_OOM; return nullptr; }
      tmp.push_back(d);
      cudaMemcpyAsync(d, src, bytes, cudaMemcpyHostToDevice, c->stream);
      return d;
    };
    for (int q = 0; q < 3; ++q) {
      pd.count[q] = (q < nsub) ? pairs->count[q] : 0;
      const size_t n = static_cast<size_t>(pd.count[q] > 0 ? pd.count[q] : 0);
      if (n == 0) continue;
      if (!pairs->glA[q] && !pairs->rA[q]) { st = DVM_ERR_PARAM; break; }
      if ((pairs->glA[q] && !pairs->glB[q]) || (!pairs->glA[q] && !pairs->rB[q])) {
        st = DVM_ERR_PARAM;
        break;
      }
      if (!pairs->r_phi[q] || !pairs->r_cos[q]) { st = DVM_ERR_PARAM; break; }
      pd.glA[q] = static_cast<const int*>(up(pairs->glA[q], n * sizeof(int)));
      pd.glB[q] = static_cast<const int*>(up(pairs->glB[q], n * sizeof(int)));
      pd.rA[q] = static_cast<const double*>(up(pairs->rA[q], n * sizeof(double)));
      pd.rB[q] = static_cast<const double*>(up(pairs->rB[q], n * sizeof(double)));
      pd.rphi[q] = static_cast<const double*>(up(pairs->r_phi[q], n * NR * sizeof(double)));
      pd.rcos[q] = static_cast<const double*>(up(pairs->r_cos[q], n * NR * sizeof(double)));
      if (pairs->glA[q]) {
        // node indices must lie on the grid
        std::vector<int> chk(pairs->glA[q], pairs->glA[q] + n);
        chk.insert(chk.end(), pairs->glB[q], pairs->glB[q] + n);
        for (int v : chk)
          if (v < 0 || v >= c->g.nv) { st = DVM_ERR_PARAM; break; }
      }
    }
  }
  if (!st) {
    CdfArgs ca{};
    ca.g = c->g; ca.cp = coll_params(c); ca.ncells = c->ncells;
    ca.f = c->d_f; ca.props = c->d_props; ca.eq_cache = c->d_eq_cache;
    ca.cum_eq = c->d_cum_eq; ca.cum_dev = c->d_cum_dev;
    ca.ref_eq = c->d_ref_eq; ca.ref_dev = c->d_ref_dev; ca.plan = c->d_plan;
    ca.pairs = pd; ca.err = c->d_err;
    st = launch(c, DVM_K_CDF, [&] { return launch_cdf(ca, c->stream); });
  }
  if (!st)
    st = launch(c, DVM_K_PLAN, [&] {
      const int grid = (c->p.precision == DVM_PREC_FP32) ? c->collide_f32_grid : c->collide_grid;
      return launch_plan(c->ncells, c->d_plan, c->d_chunk_off, c->d_total_samples,
                         static_cast<long long>(grid) * (kCollideChunk / 32), c->stream);
    });
  if (!st) {
    CollideArgs a{};
    a.g = c->g; a.cp = coll_params(c); a.t = c->tabs; a.ncells = c->ncells;
    a.step = static_cast<uint32_t>(step);
    a.step_dev = c->step_dev;
    a.f = c->d_f; a.cum_eq = c->d_cum_eq; a.cum_dev = c->d_cum_dev;
    a.ref_eq = c->d_ref_eq; a.ref_dev = c->d_ref_dev; a.plan = c->d_plan;
    a.chunk_off = c->d_chunk_off; a.pairs = pd; a.err = c->d_err;
    // d_total_samples[1]: the adds into f (df) of this call
    a.scatter_count = reinterpret_cast<unsigned long long*>(c->d_total_samples + 1);
    st = cuda_status(cudaMemsetAsync(a.scatter_count, 0, sizeof(unsigned long long), c->stream));
    if (!st && c->p.precision == DVM_PREC_FP32) {
      st = launch(c, DVM_K_COLLIDE, [&] {
        return launch_collide_f32(a, c->tabs_f, c->d_df, c->collide_f32_grid, c->stream);
      });
      if (!st) {
        ProjectArgs pa{c->g, c->ncells, c->d_f, c->d_df, c->d_props};
        st = launch(c, DVM_K_PROJECT, [&] { return launch_project(pa, c->stream); });
      }
    } else if (!st) {
      st = launch(c, DVM_K_COLLIDE, [&] { return launch_collide(a, c->collide_grid, c->stream); });
    }
  }
  if (!tmp.empty()) {
    cudaStreamSynchronize(c->stream);
    for (void* d : tmp) cudaFree(d);
  }
  return st;
}

int dvm_compute_convection(dvm_ctx* c) {
  if (!c) return DVM_ERR_PARAM;
  if (c->p.conv_method == DVM_CONV_NONE) return DVM_OK;
  int st = DVM_OK;
  if (c->p.geometry == DVM_GEOM_2D) {
    WallArgs w{};
    w.g = c->g; w.nxs = c->p.nx_space; w.nys = c->p.ny_space;
    for (int s = 0; s < 4; ++s) w.base[s] = c->wall_base[s];
    w.nentries = c->wall_entries;
    w.acc = c->p.acc_coeff; w.mass = c->p.mass; w.pi = c->pi;
    std::memcpy(w.wall, c->p.wall, sizeof(w.wall));
    w.f = c->d_f; w.ghost = c->d_ghost; w.err = c->d_err;
    st = launch(c, DVM_K_WALL, [&] { return launch_wall_flux(w, c->stream); });
    if (!st) st = launch(c, DVM_K_GHOST, [&] { return launch_wall_specular(w, c->stream); });
    if (!st) {
      Convect2DArgs a{};
      a.g = c->g; a.nxs = c->p.nx_space; a.nys = c->p.ny_space;
      a.bc_left = c->p.bc[DVM_WALL_LEFT]; a.bc_right = c->p.bc[DVM_WALL_RIGHT];
      for (int s = 0; s < 4; ++s) a.base[s] = c->wall_base[s];
      a.xf = c->p.dt / c->p.dx; a.yf = c->p.dt / c->p.dy;
      a.cfl = c->d_cfl;
      a.f = c->d_f; a.ghost = c->d_ghost; a.fconv = c->d_fconv;
      st = launch(c, DVM_K_CONVECT, [&] { return launch_convect2d(a, c->ncells, c->stream); });
    }
  } else {
    Convect1DArgs a{};
    a.g = c->g; a.nxs = c->p.nx_space; a.rows = c->p.ny_space;
    a.bc[0] = c->p.bc[DVM_WALL_LEFT]; a.bc[1] = c->p.bc[DVM_WALL_RIGHT];
    a.factor = c->p.dt / c->p.dx;
    a.acc = c->p.acc_coeff; a.mass = c->p.mass; a.pi = c->pi;
    std::memcpy(a.wall[0], c->p.wall[DVM_WALL_LEFT], sizeof(a.wall[0]));
    std::memcpy(a.wall[1], c->p.wall[DVM_WALL_RIGHT], sizeof(a.wall[1]));
    a.f = c->d_f; a.fconv = c->d_fconv; a.err = c->d_err;
    st = launch(c, DVM_K_CONVECT, [&] { return launch_convect1d(a, c->stream); });
    const bool nodes = (a.bc[0] != DVM_BC1D_DIFFUSE) || (a.bc[1] != DVM_BC1D_DIFFUSE);
    const bool diffuse = (a.bc[0] == DVM_BC1D_DIFFUSE) || (a.bc[1] == DVM_BC1D_DIFFUSE);
    if (!st && nodes) st = launch(c, DVM_K_BC1D, [&] { return launch_bc1d_nodes(a, c->stream); });
    if (!st && diffuse) st = launch(c, DVM_K_BC1D, [&] { return launch_bc1d(a, c->stream); });
  }
  if (!st) std::swap(c->d_f, c->d_fconv);  // perform_dist_func_update (phi <- phi_conv)
  return st;
}

int dvm_step(dvm_ctx* c, uint64_t first_step, int nsteps) {
  if (!c || nsteps < 0) return DVM_ERR_PARAM;
  for (int s = 0; s < nsteps; ++s) {
    int st = dvm_compute_collision_integral(c, first_step + static_cast<uint64_t>(s), nullptr);
    if (!st) st = dvm_compute_convection(c);
    if (!st) st = dvm_calculate_physical_properties(c);
    if (st) return st;
  }
  return DVM_OK;
}

int dvm_step_host(dvm_ctx* c, uint64_t first_step, int nsteps, const double* f_in,
                  double* f_out) {
  if (!c || !f_in || !f_out || nsteps < 1) return DVM_ERR_PARAM;
  // the device's view of a page-locked host buffer (null if the device cannot reach it)
  auto device_view = [](const void* p) -> void* {
    cudaPointerAttributes at{};
    if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
      cudaGetLastError();
      return nullptr;
    }
    if (at.type == cudaMemoryTypeHost || at.type == cudaMemoryTypeManaged) return at.devicePointer;
    return nullptr;
  };
  const double* din = static_cast<const double*>(device_view(f_in));
  double* dout = static_cast<double*>(device_view(f_out));
  int st = DVM_OK;
  if (din) {
    // the moments of the new state, read from host memory, write the device's copy of f
    MomentArgs a{c->g, c->ncells, c->p.mass, din, c->d_props, c->d_err, c->d_residual, c->d_f};
    st = cuda_status(cudaMemsetAsync(c->d_residual, 0, sizeof(unsigned long long), c->stream));
    if (!st) st = launch(c, DVM_K_MOMENTS, [&] { return launch_moments(a, c->stream); });
  } else {
    st = dvm_upload_f(c, f_in);
  }
  for (int s = 0; s < nsteps && !st; ++s) {
    st = dvm_compute_collision_integral(c, first_step + static_cast<uint64_t>(s), nullptr);
    if (!st) st = dvm_compute_convection(c);
    if (st) break;
    if (s + 1 < nsteps || !dout) {
      st = dvm_calculate_physical_properties(c);
    } else {
      // the last moments write the result to host memory as they read it
      MomentArgs a{c->g, c->ncells, c->p.mass, c->d_f, c->d_props, c->d_err, c->d_residual,
                   dout};
      st = cuda_status(cudaMemsetAsync(c->d_residual, 0, sizeof(unsigned long long), c->stream));
      if (!st) st = launch(c, DVM_K_MOMENTS, [&] { return launch_moments(a, c->stream); });
    }
  }
  if (!st && !dout) {
    const size_t bytes = static_cast<size_t>(c->ncells) * c->g.nv * sizeof(double);
    st = cuda_status(cudaMemcpyAsync(f_out, c->d_f, bytes, cudaMemcpyDeviceToHost, c->stream));
  }
  if (st) return st;
  return cuda_status(cudaStreamSynchronize(c->stream));
}

int dvm_last_collision_count(dvm_ctx* c, int64_t* count) {
  if (!c || !count) return DVM_ERR_PARAM;
  if (!c->d_total_samples) { *count = 0; return DVM_OK; }
  long long v = 0;
  int st = cuda_status(cudaMemcpyAsync(&v, c->d_total_samples, sizeof(v), cudaMemcpyDeviceToHost,
                                       c->stream));
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream));
  *count = v;
  return st;
}

int dvm_last_scatter_count(dvm_ctx* c, int64_t* count) {
  if (!c || !count) return DVM_ERR_PARAM;
  if (!c->d_total_samples) { *count = 0; return DVM_OK; }
  long long v = 0;
  int st = cuda_status(cudaMemcpyAsync(&v, c->d_total_samples + 1, sizeof(v),
                                       cudaMemcpyDeviceToHost, c->stream));
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream));
  *count = v;
  return st;
}

int dvm_synchronize(dvm_ctx* c) {
  if (!c) return DVM_ERR_PARAM;
  return cuda_status(cudaStreamSynchronize(c->stream));
}

int dvm_get_error_word(dvm_ctx* c, uint32_t* word) {
  if (!c || !word) return DVM_ERR_PARAM;
  uint32_t v = 0;
  int st = cuda_status(cudaMemcpyAsync(&v, c->d_err, sizeof(v), cudaMemcpyDeviceToHost, c->stream));
  if (!st) st = cuda_status(cudaMemsetAsync(c->d_err, 0, sizeof(uint32_t), c->stream));
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream));
  *word = v;
  return st;
}

int dvm_profile_enable(dvm_ctx* c, int enable) {
  if (!c) return DVM_ERR_PARAM;
  c->profile = enable != 0;
  return DVM_OK;
}

int dvm_profile_read(dvm_ctx* c, int kid, double* total_ms, int64_t* launches) {
  if (!c || kid < 0 || kid >= DVM_K_COUNT) return DVM_ERR_PARAM;
  harvest(c);
  if (total_ms) *total_ms = c->prof_ms[kid];
  if (launches) *launches = c->prof_n[kid];
  return DVM_OK;
}

int dvm_profile_reset(dvm_ctx* c) {
  if (!c) return DVM_ERR_PARAM;
  harvest(c);
  for (int k = 0; k < DVM_K_COUNT; ++k) { c->prof_ms[k] = 0.0; c->prof_n[k] = 0; }
  return DVM_OK;
}

int dvm_launch_count(dvm_ctx* c, int64_t* launches) {
  if (!c || !launches) return DVM_ERR_PARAM;
  *launches = c->launches;
  return DVM_OK;
}

int dvm_time_steps(dvm_ctx* c, uint64_t first_step, int nsteps, double* ms) {
  if (!c || !ms) return DVM_ERR_PARAM;
  cudaEvent_t a = take_event(c), b = take_event(c);
  cudaEventRecord(a, c->stream);
  int st = dvm_step(c, first_step, nsteps);
  cudaEventRecord(b, c->stream);
  if (!st) st = cuda_status(cudaEventSynchronize(b));
  float t = 0.f;
  if (!st) st = cuda_status(cudaEventElapsedTime(&t, a, b));
  *ms = t;
  c->ev_pool.push_back(a);
  c->ev_pool.push_back(b);
  return st;
}

int dvm_get_residual(dvm_ctx* c, double* residual) {
  if (!c || !residual) return DVM_ERR_PARAM;
  unsigned long long v = 0;
  int st = cuda_status(cudaMemcpyAsync(&v, c->d_residual, sizeof(v), cudaMemcpyDeviceToHost,
                                       c->stream));
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream));
  double r;
  std::memcpy(&r, &v, sizeof(r));
  *residual = r;
  return st;
}

}  // extern "C"

// ---- checkpoint / restart ------------------------------------------------------------
// Layout: a header, then f [C][Nv], the properties [C][NPROP], and with collisions the
// equilibrium cache [C][4], the cached equilibrium [C][Nv+1] with its CDF [C][Nv+1] and
// bucket table [C][1000] (the state a cache hit of the next step reuses). Everything else
// a step reads is rebuilt within the step.
namespace {
struct CkptHeader {
  char magic[8];        // "DVMCKPT2"
  uint64_t ntime;
  int32_t ncells, nv, geometry, coll_method, precision, nprop;
  uint64_t bytes;
};

struct CkptPart {
  void* dev;
  size_t bytes;
};

int ckpt_parts(dvm_ctx* c, CkptPart (&parts)[6]) {
  const size_t C = c->ncells, nv = c->g.nv;
  int n = 0;
  parts[n++] = {c->d_f, C * nv * sizeof(double)};
  parts[n++] = {c->d_props, C * DVM_NPROP * sizeof(double)};
  if (c->p.coll_method != DVM_COLL_NONE) {
    parts[n++] = {c->d_eq_cache, C * kEqCache * sizeof(double)};
    parts[n++] = {c->d_cum_eq, C * (nv + 1) * sizeof(long long)};
    parts[n++] = {c->d_ref_eq, C * kNRef * sizeof(int2)};
  }
  return n;
}
}  // namespace

extern "C" {

int dvm_checkpoint_size(dvm_ctx* c, uint64_t* bytes) {
  if (!c || !bytes) return DVM_ERR_PARAM;
  CkptPart parts[6];
  const int n = ckpt_parts(c, parts);
  uint64_t b = sizeof(CkptHeader);
  for (int i = 0; i < n; ++i) b += parts[i].bytes;
  *bytes = b;
  return DVM_OK;
}

int dvm_checkpoint_save(dvm_ctx* c, uint64_t ntime, void* buf, uint64_t bytes) {
  uint64_t need = 0;
  if (!c || !buf || dvm_checkpoint_size(c, &need) || bytes < need) return DVM_ERR_PARAM;
  CkptHeader h{};
  std::memcpy(h.magic, "DVMCKPT2", 8);
  h.ntime = ntime;
  h.ncells = c->ncells; h.nv = c->g.nv; h.geometry = c->p.geometry;
  h.coll_method = c->p.coll_method; h.precision = c->p.precision; h.nprop = DVM_NPROP;
  h.bytes = need;
  std::memcpy(buf, &h, sizeof(h));
  CkptPart parts[6];
  const int n = ckpt_parts(c, parts);
  char* p = static_cast<char*>(buf) + sizeof(h);
  int st = DVM_OK;
  for (int i = 0; i < n && !st; ++i) {
    st = cuda_status(cudaMemcpyAsync(p, parts[i].dev, parts[i].bytes, cudaMemcpyDeviceToHost,
                                     c->stream));
    p += parts[i].bytes;
  }
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream));
  return st;
}

int dvm_checkpoint_load(dvm_ctx* c, const void* buf, uint64_t bytes, uint64_t* ntime) {
  uint64_t need = 0;
  if (!c || !buf || dvm_checkpoint_size(c, &need) || bytes < need) return DVM_ERR_PARAM;
  CkptHeader h;
  std::memcpy(&h, buf, sizeof(h));
  if (std::memcmp(h.magic, "DVMCKPT2", 8) != 0 || h.bytes != need || h.ncells != c->ncells ||
      h.nv != c->g.nv || h.geometry != c->p.geometry || h.coll_method != c->p.coll_method ||
      h.nprop != DVM_NPROP)
    return DVM_ERR_PARAM;
  CkptPart parts[6];
  const int n = ckpt_parts(c, parts);
  const char* p = static_cast<const char*>(buf) + sizeof(h);
  int st = DVM_OK;
  for (int i = 0; i < n && !st; ++i) {
    st = cuda_status(cudaMemcpyAsync(parts[i].dev, p, parts[i].bytes, cudaMemcpyHostToDevice,
                                     c->stream));
    p += parts[i].bytes;
  }
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream));
  if (!st && ntime) *ntime = h.ntime;
  return st;
}

}  // extern "C"

extern "C" {

int dvm_flush_l2(dvm_ctx* c) {
  if (!c) return DVM_ERR_PARAM;
  if (!c->d_flush) {
    c->flush_n = (size_t(256) << 20) / sizeof(double);  // 256 MiB > 129 MB of L2
    int st = dalloc(c, &c->d_flush, c->flush_n);
    if (st) return st;
  }
  return cuda_status(launch_flush(c->d_flush, c->flush_n, c->stream));
}

int dvm_wait_selftest(dvm_ctx* c) {
  if (!c) return DVM_ERR_PARAM;
  int st = cuda_status(launch_wait_selftest(c->d_err, c->stream));
  if (!st) st = cuda_status(cudaStreamSynchronize(c->stream));
  return st;
}

int dvm_atomic_rate(dvm_ctx* c, uint64_t window_bytes, double* per_s) {
  if (!c || !per_s || window_bytes < sizeof(double)) return DVM_ERR_PARAM;
  int st = dvm_flush_l2(c);  // allocates the scratch buffer
  if (st) return st;
  const size_t n = std::min(static_cast<size_t>(window_bytes / sizeof(double)), c->flush_n);
  const int blocks = c->num_sms * 8, per_thread = 256;
  cudaEvent_t e0 = take_event(c), e1 = take_event(c);
  st = cuda_status(launch_atomic_probe(c->d_flush, n, blocks, per_thread, c->stream));  // warm
  if (!st) cudaEventRecord(e0, c->stream);
  if (!st) st = cuda_status(launch_atomic_probe(c->d_flush, n, blocks, per_thread, c->stream));
  if (!st) cudaEventRecord(e1, c->stream);
  if (!st) st = cuda_status(cudaEventSynchronize(e1));
  float ms = 0.f;
  if (!st) cudaEventElapsedTime(&ms, e0, e1);
  c->ev_pool.push_back(e0);
  c->ev_pool.push_back(e1);
  *per_s = ms > 0.f ? static_cast<double>(blocks) * 256.0 * per_thread / (ms * 1e-3) : 0.0;
  return st;
}

}  // extern "C"

// ----------------------------------------------------------------------------------------
// Batched homogeneous instances (dvm_batch_*).
struct dvm_batch {
  std::vector<dvm_ctx*> groups;
  std::vector<int> group_grid;          // grid index of each group
  std::vector<int> inst_group, inst_cell;
  cudaStream_t stream = nullptr;
  // one step of every instance as a graph; 1-D instances swap f and f_conv every step, so
  // they take two graphs, one for each placement of f (exec[parity])
  cudaGraphExec_t exec[2] = {nullptr, nullptr};
  int parity = 0;
  bool swaps = false;        // 1-D instances with convection
  int cells_per_inst = 1;    // 0-D: 1; 1-D: the cells of one instance (a row)
  int conv_launches = 0;     // convection launches of one step (all groups)
  uint32_t* d_step = nullptr;
  bool props_stale = true;
  int64_t collisions_per_step = 0;
  // launch shape of the grouped kernels, chosen by the autotuner
  int cdf_threads = 256;
  int collide_bps = 0;   // persistent collide CTAs per SM (0: not tuned yet)
  std::vector<double> group_cost;  // collide time of each group alone (ms): the CTA shares
  std::vector<double> tune_log;  // (cdf threads | collide CTAs/SM, ms) pairs, in tuning order
};

namespace {

void batch_release(dvm_batch* b) {
  if (!b) return;
  if (b->stream) cudaStreamSynchronize(b->stream);
  for (cudaGraphExec_t& e : b->exec)
    if (e) cudaGraphExecDestroy(e);
  for (dvm_ctx* c : b->groups) release(c);
  if (b->d_step) cudaFree(b->d_step);
  if (b->stream) cudaStreamDestroy(b->stream);
  delete b;
}

// CTAs of a persistent launch dealt to the groups in proportion to their samples per step,
// at least one each: first[g] is group g's first CTA.
void partition_ctas(int total, const std::vector<double>& work, int* first) {
  const int ng = static_cast<int>(work.size());
  double W = 0.0;
  for (double w : work) W += w;
  total = std::max(total, ng);
  std::vector<int> n(ng, 1);
  int used = ng;
  std::vector<std::pair<double, int>> rem;
  for (int g = 0; g < ng; ++g) {
    const double share = W > 0.0 ? work[g] / W * total : static_cast<double>(total) / ng;
    const int extra = std::max(0, static_cast<int>(share) - 1);
    n[g] += extra;
    used += extra;
    rem.push_back({share - static_cast<double>(n[g]), g});
  }
  std::sort(rem.begin(), rem.end(), [](const std::pair<double, int>& x,
                                       const std::pair<double, int>& y) {
    return x.first > y.first || (x.first == y.first && x.second < y.second);
  });
  for (size_t k = 0; used < total && k < rem.size(); ++k, ++used) ++n[rem[k].second];
  first[0] = 0;
  for (int g = 0; g < ng; ++g) first[g + 1] = first[g] + n[g];
}

// The grouped launch records of groups [g0, g0 + ng) of a batch.
struct GroupedStep {
  GroupedCdf cdf;
  GroupedPlan plan;
  GroupedCollide col;
  GroupedProject proj;
  GroupedMoments mom;
  bool fp32;
};

void grouped_records(const dvm_batch* b, int g0, int ng, int bps, GroupedStep& gs) {
  std::memset(&gs, 0, sizeof(gs));
  gs.cdf.ngroups = gs.plan.ngroups = gs.col.ngroups = gs.proj.ngroups = gs.mom.ngroups = ng;
  gs.fp32 = (b->groups[g0]->p.precision == DVM_PREC_FP32);
  std::vector<double> work(ng);
  int cells = 0;
  for (int k = 0; k < ng; ++k) {
    const dvm_ctx* c = b->groups[g0 + k];
    gs.cdf.first[k] = gs.proj.first[k] = gs.mom.first[k] = cells;
    cells += c->ncells;
    CdfArgs& ca = gs.cdf.a[k];
    ca.g = c->g; ca.cp = coll_params(c); ca.ncells = c->ncells;
    ca.f = c->d_f; ca.props = c->d_props; ca.eq_cache = c->d_eq_cache;
    ca.cum_eq = c->d_cum_eq; ca.cum_dev = c->d_cum_dev;
    ca.ref_eq = c->d_ref_eq; ca.ref_dev = c->d_ref_dev; ca.plan = c->d_plan; ca.err = c->d_err;
    gs.plan.ncells[k] = c->ncells;
    gs.plan.plan[k] = c->d_plan;
    gs.plan.chunk_off[k] = c->d_chunk_off;
    gs.plan.total[k] = c->d_total_samples;
    CollideArgs a{};
    a.g = c->g; a.cp = coll_params(c); a.t = c->tabs; a.ncells = c->ncells;
    a.step_dev = c->step_dev;
    a.f = c->d_f; a.cum_eq = c->d_cum_eq; a.cum_dev = c->d_cum_dev;
    a.ref_eq = c->d_ref_eq; a.ref_dev = c->d_ref_dev; a.plan = c->d_plan;
    a.chunk_off = c->d_chunk_off; a.err = c->d_err;
    gs.col.a[k] = collide_consts(a);
    gs.col.tf[k] = c->tabs_f;
    gs.col.df[k] = c->d_df;
    gs.proj.a[k] = ProjectArgs{c->g, c->ncells, c->d_f, c->d_df, c->d_props};
    gs.mom.a[k] = MomentArgs{c->g, c->ncells, c->p.mass, c->d_f, c->d_props, c->d_err,
                             nullptr, nullptr};
    work[k] = b->group_cost.size() == b->groups.size()
                  ? b->group_cost[g0 + k]
                  : static_cast<double>(c->ncells) * static_cast<double>(c->p.samples_per_step);
  }
  gs.cdf.first[ng] = gs.proj.first[ng] = gs.mom.first[ng] = cells;
  partition_ctas(b->groups[g0]->num_sms * bps, work, gs.col.first);
  for (int k = 0; k < ng; ++k)
    gs.plan.warps[k] = static_cast<long long>(gs.col.first[k + 1] - gs.col.first[k]) *
                       (kCollideChunk / 32);
}

// CTAs per SM the grouped collide launch of groups [g0, g0 + ng) can hold.
int grouped_max_bps(const dvm_batch* b, int g0, int ng) {
  GroupedStep gs;
  grouped_records(b, g0, ng, 1, gs);
  return std::min(4, collide_grouped_blocks_per_sm(gs.col, gs.fp32));
}

// One step of every instance: per block of up to kMaxGroups grids, one launch each of the
// CDF build, the plan, the persistent collision kernel (the precision form adds the
// projection) and the moments.
int batch_issue(dvm_batch* b, bool cdf = true, bool plan = true, bool collide = true,
                bool moments = true) {
  const int G = static_cast<int>(b->groups.size());
  for (int g0 = 0; g0 < G; g0 += kMaxGroups) {
    const int ng = std::min(kMaxGroups, G - g0);
    const int bps = std::min(b->collide_bps > 0 ? b->collide_bps : 4, grouped_max_bps(b, g0, ng));
    GroupedStep gs;
    grouped_records(b, g0, ng, bps, gs);
    int st = DVM_OK;
    if (cdf) st = cuda_status(launch_cdf_grouped(gs.cdf, b->cdf_threads, b->stream));
    if (!st && plan) st = cuda_status(launch_plan_grouped(gs.plan, b->stream));
    if (!st && collide) {
      st = cuda_status(launch_collide_grouped(gs.col, gs.fp32, b->stream));
      if (!st && gs.fp32) st = cuda_status(launch_project_grouped(gs.proj, b->stream));
    }
    if (!st && moments && b->swaps) {
      // 1-D rows: convection and ends per group (each swaps its f and f_conv), then the
      // moments of the new f
      for (int k = 0; k < ng && !st; ++k) st = dvm_compute_convection(b->groups[g0 + k]);
      if (!st) grouped_records(b, g0, ng, bps, gs);
    }
    if (!st && moments) st = cuda_status(launch_moments_grouped(gs.mom, b->stream));
    if (st) return st;
  }
  return DVM_OK;
}

// Launch-shape autotuner for the grouped step: the CDF CTA width (256, 512, 1024 threads)
// and the persistent collide CTAs per SM (1..4, bounded by occupancy), each timed on the
// batch's own state, which is saved first (f into f_conv, unused by 0-D contexts; the
// equilibrium caches to the host) and restored afterwards.
int autotune(dvm_batch* b) {
  b->tune_log.clear();
  std::vector<std::vector<double>> caches(b->groups.size());
  int st = DVM_OK;
  for (size_t k = 0; k < b->groups.size() && !st; ++k) {
    dvm_ctx* c = b->groups[k];
    const size_t bytes = static_cast<size_t>(c->ncells) * c->g.nv * sizeof(double);
    st = cuda_status(cudaMemcpyAsync(c->d_fconv, c->d_f, bytes, cudaMemcpyDeviceToDevice,
                                     b->stream));
    caches[k].resize(static_cast<size_t>(c->ncells) * kEqCache);
    if (!st && c->d_eq_cache)
      st = cuda_status(cudaMemcpyAsync(caches[k].data(), c->d_eq_cache,
                                       caches[k].size() * sizeof(double),
                                       cudaMemcpyDeviceToHost, b->stream));
  }
  if (!st) st = cuda_status(cudaStreamSynchronize(b->stream));
  if (st) return st;
  auto restore_f = [&]() {
    for (dvm_ctx* c : b->groups) {
      const size_t bytes = static_cast<size_t>(c->ncells) * c->g.nv * sizeof(double);
      cudaMemcpyAsync(c->d_f, c->d_fconv, bytes, cudaMemcpyDeviceToDevice, b->stream);
    }
  };
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  auto timed = [&](bool cdf, bool collide, float& ms) -> int {
    for (int rep = 0; rep < 2; ++rep) {  // the first pass warms up
      if (collide) restore_f();
      cudaEventRecord(e0, b->stream);
      const int s2 = batch_issue(b, cdf, false, collide, false);
      cudaEventRecord(e1, b->stream);
      if (s2) return s2;
      const int s3 = cuda_status(cudaEventSynchronize(e1));
      if (s3) return s3;
      cudaEventElapsedTime(&ms, e0, e1);
    }
    return DVM_OK;
  };
  float best = 1e30f, ms = 0.f;
  int best_t = 256;
  for (int t : {256, 512, 1024}) {
    b->cdf_threads = t;
    st = timed(true, false, ms);
    if (st) break;
    b->tune_log.push_back(t);
    b->tune_log.push_back(ms);
    if (ms < best) { best = ms; best_t = t; }
  }
  b->cdf_threads = best_t;
  if (!st) st = batch_issue(b, true, true, false, false);  // the plan the collide walks
  // each group's collide alone on the whole GPU: its time sets the group's share of CTAs
  b->group_cost.clear();
  for (size_t g = 0; g < b->groups.size() && !st; ++g) {
    GroupedStep gs;
    grouped_records(b, static_cast<int>(g), 1, grouped_max_bps(b, static_cast<int>(g), 1), gs);
    for (int rep = 0; rep < 2 && !st; ++rep) {
      restore_f();
      cudaEventRecord(e0, b->stream);
      st = cuda_status(launch_collide_grouped(gs.col, gs.fp32, b->stream));
      cudaEventRecord(e1, b->stream);
      if (!st) st = cuda_status(cudaEventSynchronize(e1));
      if (!st) cudaEventElapsedTime(&ms, e0, e1);
    }
    b->group_cost.push_back(std::max(static_cast<double>(ms), 1e-6));
  }
  if (st) b->group_cost.clear();
  int max_bps = 4;
  for (size_t g0 = 0; g0 < b->groups.size(); g0 += kMaxGroups)
    max_bps = std::min(max_bps, grouped_max_bps(b, static_cast<int>(g0),
                                                std::min<int>(kMaxGroups, b->groups.size() - g0)));
  best = 1e30f;
  int best_b = max_bps;
  for (int bps = 1; bps <= max_bps && !st; ++bps) {
    b->collide_bps = bps;
    st = timed(false, true, ms);
    if (st) break;
    b->tune_log.push_back(bps);
    b->tune_log.push_back(ms);
    if (ms < best) { best = ms; best_b = bps; }
  }
  b->collide_bps = best_b;
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (st) return st;
  restore_f();
  for (size_t k = 0; k < b->groups.size() && !st; ++k) {
    dvm_ctx* c = b->groups[k];
    if (c->d_eq_cache)
      st = cuda_status(cudaMemcpyAsync(c->d_eq_cache, caches[k].data(),
                                       caches[k].size() * sizeof(double),
                                       cudaMemcpyHostToDevice, b->stream));
  }
  if (!st) st = cuda_status(cudaStreamSynchronize(b->stream));
  return st;
}

int batch_prepare(dvm_batch* b) {
  if (b->props_stale) {
    for (dvm_ctx* c : b->groups) {
      int st = dvm_calculate_physical_properties(c);
      if (st) return st;
    }
    int st = cuda_status(cudaStreamSynchronize(b->stream));
    if (st) return st;
    b->props_stale = false;
  }
  if (b->exec[0]) return DVM_OK;
  int st = autotune(b);
  if (st) return st;
  // one step of every group, then the step counter, captured into one graph; with 1-D
  // rows a second graph for the other placement of f (the capture of the first leaves the
  // host's f and f_conv swapped, the second swaps them back)
  b->parity = 0;
  for (int e = 0; e < (b->swaps ? 2 : 1) && !st; ++e) {
    cudaGraph_t graph = nullptr;
    st = cuda_status(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeRelaxed));
    if (st) return st;
    st = batch_issue(b);
    if (!st) st = cuda_status(launch_step_end(b->d_step, nullptr, nullptr, b->stream));
    const int st2 = cuda_status(cudaStreamEndCapture(b->stream, &graph));
    if (!st) st = st2;
    if (!st) st = cuda_status(cudaGraphInstantiate(&b->exec[e], graph, 0));
    if (graph) cudaGraphDestroy(graph);
  }
  return st;
}

// Launches one step's graph and keeps the host's view of each 1-D group's f in step.
int batch_launch(dvm_batch* b) {
  const int st = cuda_status(cudaGraphLaunch(b->exec[b->parity], b->stream));
  if (st || !b->swaps) return st;
  for (dvm_ctx* c : b->groups) std::swap(c->d_f, c->d_fconv);
  b->parity ^= 1;
  return DVM_OK;
}

}  // namespace

namespace dvm {

int ctx_create(const dvm_params* p, const dvm_vgrid* vg, bool async_alloc, dvm_ctx** out) {
  return create_context(p, vg, nullptr, async_alloc, out);
}
void ctx_destroy(dvm_ctx* c) { release(c); }
cudaStream_t ctx_stream(const dvm_ctx* c) { return c->stream; }
const unsigned long long* ctx_residual(const dvm_ctx* c) { return c->d_residual; }
const long long* ctx_total_samples(const dvm_ctx* c) { return c->d_total_samples; }
void ctx_set_step_dev(dvm_ctx* c, const uint32_t* step) { c->step_dev = step; }
size_t ctx_device_bytes(const dvm_ctx* c) { return c->device_bytes; }

size_t context_bytes(const dvm_params* p, const dvm_vgrid* vg) {
  const size_t C = static_cast<size_t>(p->nx_space) * p->ny_space;
  const size_t nv = static_cast<size_t>(vg->nx) * vg->ny * vg->nz;
  const size_t d = sizeof(double);
  size_t b = 2 * (vg->nx + vg->ny + vg->nz) * d            // axes
             + 2 * C * nv * d + C * DVM_NPROP * d           // f, f_conv, properties
             + sizeof(uint32_t) + nv * sizeof(float2)       // error word, speeds
             + sizeof(unsigned long long);                  // residual
  if (p->coll_method != DVM_COLL_NONE) {
    b += 2 * C * (nv + 1) * d   // cum_eq, cum_dev
         + C * kEqCache * d;      // equilibrium cache
    b += 2 * C * kNRef * sizeof(int2) + C * sizeof(CellPlan) +
         (3 * C + 1) * sizeof(long long) + 2 * sizeof(long long);
    const size_t nmax = std::max(vg->nx, std::max(vg->ny, vg->nz));
    b += 3 * nmax * sizeof(AxisEntry) + kTrigN * sizeof(double2);
    const bool cubic = (vg->nx == vg->ny && vg->ny == vg->nz);
    const size_t ns = cubic ? 3 * static_cast<size_t>(vg->nx - 1) * (vg->nx - 1) + 1 : 0;
    b += ns * sizeof(double2);
    if (p->precision == DVM_PREC_FP32)
      b += 3 * nmax * sizeof(AxisEntryF) + kTrigN * sizeof(float2) + ns * sizeof(float2) +
           C * nv * sizeof(float);
  }
  if (p->geometry == DVM_GEOM_2D && p->conv_method == DVM_CONV_UPWIND1) {
    size_t n = 2 * static_cast<size_t>(p->nx_space);
    if (p->bc[DVM_WALL_LEFT] == DVM_BC2D_WALL) n += p->ny_space;
    if (p->bc[DVM_WALL_RIGHT] == DVM_BC2D_WALL) n += p->ny_space;
    b += n * nv * d + static_cast<size_t>(vg->nx + vg->ny) * sizeof(float2);
  }
  return b;
}

}  // namespace dvm

extern "C" {

int dvm_footprint_bytes(const dvm_params* params, const dvm_vgrid* vgrid, uint64_t* bytes) {
  if (!bytes) return DVM_ERR_PARAM;
  const int st = validate(params, vgrid);
  if (st) return st;
  *bytes = dvm::context_bytes(params, vgrid);
  return DVM_OK;
}

int dvm_batch_create(const dvm_params* params, const dvm_vgrid* grids, int ngrids,
                     const int32_t* instance_grid, int ninstances,
                     const int64_t* samples_per_grid, dvm_batch** out) {
  if (!params || !grids || !instance_grid || !samples_per_grid || !out || ngrids < 1 ||
      ninstances < 1)
    return DVM_ERR_PARAM;
  if (params->coll_method == DVM_COLL_NONE) return DVM_ERR_PARAM;
  // 0-D instances, or 1-D instances of nx_space cells (ny_space is set per grid)
  if (params->geometry == DVM_GEOM_2D) return DVM_ERR_PARAM;
  if (params->geometry == DVM_GEOM_1D && params->nx_space < 3) return DVM_ERR_PARAM;
  *out = nullptr;
  for (int i = 0; i < ninstances; ++i)
    if (instance_grid[i] < 0 || instance_grid[i] >= ngrids) return DVM_ERR_PARAM;
  dvm_batch* b = new (std::nothrow) dvm_batch();
  if (!b) return DVM_ERR_OOM;
  if (params->geometry == DVM_GEOM_1D) {
    b->cells_per_inst = params->nx_space;
    b->swaps = (params->conv_method != DVM_CONV_NONE);
  }
  int st = cuda_status(cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking));
  if (!st) st = dalloc(&b->d_step, 1);
  if (!st) st = cuda_status(cudaMemset(b->d_step, 0, sizeof(uint32_t)));
  if (st) { batch_release(b); return st; }
  b->inst_group.assign(ninstances, -1);
  b->inst_cell.assign(ninstances, -1);
  for (int gidx = 0; gidx < ngrids; ++gidx) {
    int count = 0;
    for (int i = 0; i < ninstances; ++i)
      if (instance_grid[i] == gidx) {
        b->inst_group[i] = static_cast<int>(b->groups.size());
        b->inst_cell[i] = count++;
      }
    if (count == 0) continue;
    dvm_params p = *params;
    if (params->geometry == DVM_GEOM_1D) {
      // one row of nx_space cells per instance, each with the ends of params
      p.ny_space = count;
    } else {
      p.geometry = DVM_GEOM_0D;
      p.nx_space = count;
      p.ny_space = 1;
      p.conv_method = DVM_CONV_NONE;
    }
    p.samples_mode = DVM_SAMPLES_FIXED;
    p.samples_per_step = samples_per_grid[gidx];
    dvm_ctx* c = nullptr;
    st = create_context(&p, &grids[gidx], b->stream, false, &c);
    if (st) { batch_release(b); return st; }
    c->step_dev = b->d_step;
    b->groups.push_back(c);
    b->group_grid.push_back(gidx);
    b->collisions_per_step +=
        static_cast<int64_t>(count) * b->cells_per_inst * samples_per_grid[gidx];
    if (b->swaps) {
      // the convection of a step: the interior sweep, then the node-local and the diffuse
      // end launches its end conditions need
      const bool nodes = p.bc[DVM_WALL_LEFT] != DVM_BC1D_DIFFUSE ||
                         p.bc[DVM_WALL_RIGHT] != DVM_BC1D_DIFFUSE;
      const bool diffuse = p.bc[DVM_WALL_LEFT] == DVM_BC1D_DIFFUSE ||
                           p.bc[DVM_WALL_RIGHT] == DVM_BC1D_DIFFUSE;
      b->conv_launches += 1 + (nodes ? 1 : 0) + (diffuse ? 1 : 0);
    }
  }
  *out = b;
  return DVM_OK;
}

int dvm_batch_destroy(dvm_batch* b) {
  if (!b) return DVM_ERR_PARAM;
  batch_release(b);
  return DVM_OK;
}

int dvm_batch_upload_f(dvm_batch* b, int instance, const double* f) {
  if (!b || !f || instance < 0 || instance >= static_cast<int>(b->inst_group.size()))
    return DVM_ERR_PARAM;
  dvm_ctx* c = b->groups[b->inst_group[instance]];
  const size_t n = static_cast<size_t>(b->cells_per_inst) * c->g.nv;
  int st = cuda_status(cudaMemcpyAsync(c->d_f + b->inst_cell[instance] * n, f,
                                       n * sizeof(double), cudaMemcpyHostToDevice, b->stream));
  if (!st) st = cuda_status(cudaStreamSynchronize(b->stream));
  b->props_stale = true;
  return st;
}

int dvm_batch_download_f(dvm_batch* b, int instance, double* f) {
  if (!b || !f || instance < 0 || instance >= static_cast<int>(b->inst_group.size()))
    return DVM_ERR_PARAM;
  dvm_ctx* c = b->groups[b->inst_group[instance]];
  const size_t n = static_cast<size_t>(b->cells_per_inst) * c->g.nv;
  int st = cuda_status(cudaMemcpyAsync(f, c->d_f + b->inst_cell[instance] * n,
                                       n * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
  if (!st) st = cuda_status(cudaStreamSynchronize(b->stream));
  return st;
}

int dvm_batch_step(dvm_batch* b, int nsteps) {
  if (!b || nsteps < 0) return DVM_ERR_PARAM;
  int st = batch_prepare(b);
  if (st) return st;
  for (int s = 0; s < nsteps; ++s) {
    st = batch_launch(b);
    if (st) return st;
  }
  return DVM_OK;
}

int dvm_batch_get_properties(dvm_batch* b, double* props) {
  if (!b || !props) return DVM_ERR_PARAM;
  int st = cuda_status(cudaStreamSynchronize(b->stream));
  if (st) return st;
  const size_t n = static_cast<size_t>(b->cells_per_inst) * DVM_NPROP;
  for (size_t i = 0; i < b->inst_group.size(); ++i) {
    dvm_ctx* c = b->groups[b->inst_group[i]];
    st = cuda_status(cudaMemcpy(props + i * n, c->d_props + b->inst_cell[i] * n,
                                n * sizeof(double), cudaMemcpyDeviceToHost));
    if (st) return st;
  }
  return DVM_OK;
}

int dvm_batch_launch_shape(dvm_batch* b, int* cdf_threads, int* collide_ctas_per_sm,
                           int* launches_per_step) {
  if (!b || !cdf_threads || !collide_ctas_per_sm || !launches_per_step) return DVM_ERR_PARAM;
  const bool tuned = b->exec[0] != nullptr;
  const int blocks = (static_cast<int>(b->groups.size()) + kMaxGroups - 1) / kMaxGroups;
  const bool fp32 = !b->groups.empty() && b->groups[0]->p.precision == DVM_PREC_FP32;
  *cdf_threads = tuned ? b->cdf_threads : 0;
  *collide_ctas_per_sm = tuned ? b->collide_bps : 0;
  // per block of grids: CDF, plan, collide (+ projection), moments; the convection of 1-D
  // rows, per grid; then the step counter
  *launches_per_step = tuned ? blocks * (fp32 ? 5 : 4) + b->conv_launches + 1 : 0;
  return DVM_OK;
}

int dvm_batch_time_steps(dvm_batch* b, int nsteps, double* ms, int64_t* collisions) {
  if (!b || !ms || nsteps < 0) return DVM_ERR_PARAM;
  int st = batch_prepare(b);
  if (st) return st;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  cudaEventRecord(e0, b->stream);
  for (int s = 0; s < nsteps && !st; ++s) st = batch_launch(b);
  cudaEventRecord(e1, b->stream);
  if (!st) st = cuda_status(cudaEventSynchronize(e1));
  float t = 0.f;
  if (!st) cudaEventElapsedTime(&t, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  *ms = t;
  if (collisions) *collisions = b->collisions_per_step * nsteps;
  return st;
}

}  // extern "C"
