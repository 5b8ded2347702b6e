// dvm_kernels.cu -- sm_103a kernels of the DVM time step.
//
//   k_cdf        per-cell CDF build          compute_cdf_vr / compute_cdf_fmc
//   k_plan       sample counts -> chunk map  compute_num_coll_pairs
//   k_collide    Monte Carlo collisions      variance_reduction_kernel / full_monte_carlo_kernel
//   k_wall_flux  2-D diffuse wall ghosts     set_boundary_nodes (diffuse part)
//   k_wall_spec  2-D specular wall ghosts    set_boundary_nodes (specular part)
//   k_convect2d  2-D upwind update           first_order_scheme + ghost update
//   k_convect1d  1-D upwind update           grid_ref first_order_scheme
//   k_bc1d       1-D end conditions          grid_ref apply_boundary_conditions
//   k_moments    per-cell moments            calculate_physical_properties (+ q, tau)
//
// Layout f[cell][v], FP64. Collision contributions are scattered straight into f with
// FP64 atomics: in the monatomic step the sampling reads only the CDFs built at the start
// of the cell-step, so delta_phi = phi + sum(contributions) needs no copy of phi.
#include <cooperative_groups.h>
#include <cuda_runtime.h>

#include "dfloat.cuh"
#include "dvm_internal.h"

namespace dvm {

// ----------------------------------------------------------------------------------------
// k_cdf: one CTA per cell.
// VR: collisions/variance_reduction.f90:234-496. FMC: collisions/full_mc.f90:110-180.
//
// The cumulative sums are kept in 64-bit fixed point: every term (f_eq, |f - f_eq| or |f|,
// all nonnegative) is truncated to a multiple of 2^-k, with 2^k chosen per cell so that
// 16 n 2^k <= 2^62 (n the cell density), and summed in integers. The sums are exact and
// independent of the order of summation, so the parallel scan gives the sequential sum
// bit for bit; the quantum 2^-k is below 1e-17 n, finer than the FP64 rounding of the
// reference's running sum. The partner search (k_collide) then compares integers only.
constexpr int kCdfPer = 4;
constexpr int kCdfPitch = kCdfPer + 1;  // padded row of a lane's values in the transpose
constexpr int kCdfTrWarp = 2 * 32 * kCdfPitch;  // words per warp
constexpr int kCdfCoarseMax = 512;   // entries of the shared-memory coarse index per table

// compute_num_coll_pairs, collisions/collision_utilities.f90:106-140 (n = m); ct is
// (0.5 (T + T))^(2/3), formed once per cell, and cp.b3 the pair's mass-weighted beta3_min.
__device__ long long num_coll_pairs(const CollParams& cp, double ct, double densA,
                                    double densB) {
  const double rms_sq = cp.coln_rms * cp.coln_rms;
  const double val = (0.5 * cp.dt * ct * densA * densB) / (cp.Kn * rms_sq * cp.b3);
  if (!(val < 9.0e18)) return 0;
  return llround(val);
}

// |x| 2^k truncated to an integer, from the bits of x (no FP64 op). Terms that would not
// fit below 2^62 are clamped to 2^58 and reported; zero and FP64 subnormals give 0.
// Without branches: the 53-bit significand is placed at bit 9 (a 62-bit integer) and
// shifted right by 9 - sh, clamped to 63, which leaves 0 for every sh <= -54.
__device__ __forceinline__ long long to_fixed(double x, int k, uint32_t& bad) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(x)) &
                               0x7fffffffffffffffull;
  const int e = static_cast<int>(b >> 52);
  const int sh = e - 1075 + k;
  const unsigned long long mant = ((b & ((1ull << 52) - 1)) | (1ull << 52)) << 9;
  const int rs = min(max(9 - sh, 0), 63);
  long long r = static_cast<long long>(mant >> rs);
  if (e == 0) return 0;  // zero or FP64 subnormal
  if (e == 2047 || sh > 9) { bad |= DVM_EW_NONFINITE; r = 1ll << 58; }
  return r;
}

// x 2^k truncated towards zero, signed, for a double x (bit operations only).
__device__ __forceinline__ long long to_fixed_s(double x, int k, uint32_t& bad) {
  const long long sg = __double_as_longlong(x) >> 63;  // 0 or -1
  const long long v = to_fixed(x, k, bad);              // |x| 2^k
  return (v ^ sg) - sg;
}

// v 2^k truncated towards zero, signed, for a float v (bit operations only).
__device__ __forceinline__ long long to_fixed_f(float v, int k, uint32_t& bad) {
  const uint32_t b = static_cast<uint32_t>(__float_as_int(v));
  const int e = static_cast<int>((b >> 23) & 0xffu);
  if (e == 0) return 0;  // zero or FP32 subnormal (below 1.2e-38)
  if (e == 255) { bad |= DVM_EW_NONFINITE; return 0; }
  const unsigned long long m = (b & 0x7fffffu) | 0x800000u;
  const int sh = e - 150 + k;
  unsigned long long r;
  if (sh >= 0) {
    if (sh > 38) { bad |= DVM_EW_NONFINITE; return 0; }
    r = m << sh;
  } else {
    r = (sh <= -64) ? 0ull : (m >> (-sh));
  }
  return (b >> 31) ? -static_cast<long long>(r) : static_cast<long long>(r);
}


// to_fixed_f through the FP32 multiplier, for a scale 2^k = s1 s2 with s1, s2 normal
// powers of two: v s1 s2 is exact (flushing to zero drops only values below 2^-126, whose
// truncation is 0, and a subnormal v gives 0 as above), |v| 2^k >= 2^62 is exactly the
// overflow of to_fixed_f, and the conversion truncates towards zero.
__device__ __forceinline__ long long to_fixed_f_mul(float v, float s1, float s2,
                                                    uint32_t& bad) {
  float p;
  asm("mul.rn.ftz.f32 %0, %1, %2;" : "=f"(p) : "f"(v), "f"(s1));
  asm("mul.rn.ftz.f32 %0, %0, %1;" : "+f"(p) : "f"(s2));
  if (!(fabsf(p) < 0x1p62f)) { bad |= DVM_EW_NONFINITE; return 0; }
  return __float2ll_rz(p);
}

// Quotient n / d for 0 <= n < 2^22 (every node index: at most 128^3 nodes) from the float
// reciprocal rd = 1/d: n is formed exactly by the FP32 adder, n rd lies within 2^-23
// relative of n / d, so its truncation is the quotient or one below it, and one integer
// step corrects it (no integer division sequence, no conversion instruction).
static_assert(kMaxAxis * kMaxAxis * kMaxAxis < (1 << 22), "node indices must stay below 2^22");
__device__ __forceinline__ int quot_small(int n, int d, float rd) {
  const float nf = __fsub_rn(__int_as_float(0x4B000000 | n), 8388608.f);
  int q = __float_as_int(__fadd_rz(__fmul_rn(nf, rd), 8388608.f)) - 0x4B000000;
  if (n - q * d >= d) ++q;
  return q;
}

// (i, j, k) of node l on an NX x NY x NZ grid, with the reciprocals of NX and NX NY.
__device__ __forceinline__ void node_ijk(int l, int NX, int NXY, float rNX, float rNXY, int& i,
                                         int& j, int& k) {
  k = quot_small(l, NXY, rNXY);
  const int r = l - k * NXY;
  j = quot_small(r, NX, rNX);
  i = r - j * NX;
}

static int sm_count() {
  static int n = 0;
  if (n == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n < 1)
      n = 1;
    cudaGetLastError();
  }
  return n;
}

// Block-wide exclusive scan of two int64 per thread; tot gets the block totals.
__device__ __forceinline__ void block_scan2_i64(long long& a, long long& b, long long& tot_a,
                                                long long& tot_b, long long* s_scan) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
  long long ia = a, ib = b;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const long long ta = __shfl_up_sync(0xffffffffu, ia, o);
    const long long tb = __shfl_up_sync(0xffffffffu, ib, o);
    if (lane >= o) { ia += ta; ib += tb; }
  }
  if (lane == 31) { s_scan[warp] = ia; s_scan[32 + warp] = ib; }
  __syncthreads();
  if (warp == 0) {
    long long wa = lane < nw ? s_scan[lane] : 0, wb = lane < nw ? s_scan[32 + lane] : 0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long ta = __shfl_up_sync(0xffffffffu, wa, o);
      const long long tb = __shfl_up_sync(0xffffffffu, wb, o);
      if (lane >= o) { wa += ta; wb += tb; }
    }
    s_scan[64 + lane] = wa;
    s_scan[96 + lane] = wb;
  }
  __syncthreads();
  const long long wpa = warp > 0 ? s_scan[64 + warp - 1] : 0;
  const long long wpb = warp > 0 ? s_scan[96 + warp - 1] : 0;
  tot_a = s_scan[64 + nw - 1];
  tot_b = s_scan[96 + nw - 1];
  a = wpa + ia - a;  // exclusive
  b = wpb + ib - b;
}

// T threads per CTA (256, or 512 / 1024 for launches of few cells: the per-cell scan then
// walks fewer, wider chunks).
template <int T>
__device__ __forceinline__ void cdf_cta(const CdfArgs& a, const int cell) {
  constexpr int kCdfThreads = T;
  constexpr int kCdfChunk = T * kCdfPer;  // nodes per scan chunk
  __shared__ long long s_scan[2][128];
  __shared__ double s_par[6];
  __shared__ int s_new, s_k, s_ke;
  __shared__ dfl s_fac[3 * kMaxAxis];
  __shared__ long long s_coarse[2][kCdfCoarseMax + 1];
  __shared__ int s_right[2][kNRef];  // bucket boundaries right(r) of the two tables
  // per warp: its 4 x 32 cumulative values of both CDFs (signs in the low bits), transposed so that every
  // store instruction writes 32 consecutive positions
  extern __shared__ __align__(16) long long s_tr[];  // (T / 32) * kCdfTrWarp words
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  long long* tr_e = s_tr + warp * kCdfTrWarp;
  long long* tr_d = tr_e + 32 * kCdfPitch;
  const GridInfo& g = a.g;
  const int nv = g.nv;
  const size_t cs = static_cast<size_t>(cell) * (nv + 1);
  const double* f = a.f + static_cast<size_t>(cell) * nv;
  const double* P = a.props + static_cast<size_t>(cell) * DVM_NPROP;
  long long* ce = a.cum_eq + cs;
  long long* cd = a.cum_dev + cs;
  const bool vr = (a.cp.method == DVM_COLL_VR);
  const int NX = g.nx, NXY = g.nx * g.ny;
  // coarse index: every cstep-th cumulative value, cstep a power of two
  int cstep = 8;
  while ((nv + 1) / cstep > kCdfCoarseMax) cstep <<= 1;
  const int ncoarse = nv / cstep;  // entries 0..ncoarse

  if (threadIdx.x == 0) {
    // fixed-point scale from a density: 16 n 2^k <= 2^62
    auto scale = [](double n0) {
      int E = 1;
      if (n0 > 0.0 && isfinite(n0)) E = ilogb(n0) + 1;  // n0 < 2^E
      return 58 - E;
    };
    s_k = scale(P[DVM_P_DENS]);
    s_new = 0;
    if (vr) {
      const double dens = P[DVM_P_DENS], u = P[DVM_P_U], v = P[DVM_P_V], w = P[DVM_P_W];
      double temp = P[DVM_P_SPECIES_TEMP];
      if (temp < kDoubleTol) temp = P[DVM_P_TEMP];
      double* cache = a.eq_cache + static_cast<size_t>(cell) * kEqCache;
      const double tol = a.cp.cdf_tolerance;
      // new_eq_flag, variance_reduction.f90:316-322 (w is not tested; it is kept with the
      // cache because the cached equilibrium was built with it)
      const int nw = (fabs(dens - cache[0]) > tol * dens || fabs(u - cache[1]) > tol * u ||
                      fabs(v - cache[2]) > tol * v || fabs(temp - cache[3]) > tol * temp);
      if (nw) { cache[0] = dens; cache[1] = u; cache[2] = v; cache[3] = temp; cache[4] = w; }
      s_new = nw;
      // the equilibrium CDF keeps the scale of the density it was built for, so a cached
      // one stays valid (with its bucket table) until the cache is renewed
      s_ke = scale(cache[0]);
      // the equilibrium of the cache's moments: on a renewal the current ones; otherwise
      // the node values are formed again, bit for bit those of the renewal step
      const double cd = cache[0], ct = cache[3];
      s_par[0] = (cd > 0.0) ? cd * maxwell_coeff(a.cp.mass, ct, a.cp.pi) : 0.0;
      s_par[1] = cache[1]; s_par[2] = cache[2]; s_par[3] = cache[4]; s_par[4] = ct;
    }
  }
  __syncthreads();
  const bool recompute = vr && s_new;
  if (vr) {
    // the Maxwellian times the node volume factorises over the axes:
    // mc exp(-m|c-u|^2/T) bx by bz = [mc e_x bx] [e_y by] [e_z bz]
    const double mc = s_par[0], temp = s_par[4], m = a.cp.mass;
    const int nsum = g.nx + g.ny + g.nz;
    for (int t = threadIdx.x; t < nsum; t += blockDim.x) {
      double val = 0.0;
      if (temp > 0.0) {
        if (t < g.nx) {
          const double c = g.x[t] - s_par[1];
          val = mc * exp(-(c * c) * m / temp) * g.bx[t];
        } else if (t < g.nx + g.ny) {
          const double c = g.y[t - g.nx] - s_par[2];
          val = exp(-(c * c) * m / temp) * g.by[t - g.nx];
        } else {
          const double c = g.z[t - g.nx - g.ny] - s_par[3];
          val = exp(-(c * c) * m / temp) * g.bz[t - g.nx - g.ny];
        }
      }
      const dfl v = dfl_from_double(val);
      s_fac[t < g.nx ? t : (t < g.nx + g.ny ? kMaxAxis + t - g.nx
                                              : 2 * kMaxAxis + t - g.nx - g.ny)] =
          dfl_norm(v.hi, v.lo);
    }
    __syncthreads();
  }
  const int k = s_k, ke = s_ke;
  uint32_t bad = 0;
  // deviation and CDFs (cumul_df of variance_reduction.f90:454-456, full_mc.f90:151-152):
  // each thread takes kCdfPer consecutive nodes of a chunk, forms and scans them in
  // sequence, and the thread sums are scanned across the block. f is read straight into
  // registers as 16-byte pairs (8-byte reads where a cell's slab is not 16-byte aligned),
  // one chunk ahead of the one being scanned.
  // The node terms are formed without FP64 instructions: f enters the fixed point from
  // its bits, f_eq = e_x e_y e_z is a pair product converted to fixed point, and f - f_eq
  // and its magnitude are integer operations. For VR every term
  // uses the scale of the cached equilibrium's density (the cache is renewed whenever
  // the density moves by more than cdf_tolerance, well inside the scale's 16x margin).
  const int kc = vr ? ke : k;
  // the equilibrium's scale 2^ke as two float factors (every cell of a sane density; the
  // bit-operation conversion covers the rest)
  const bool mul_scale = (ke >= -252 && ke <= 252);
  const float s1 = mul_scale ? pow2f_exact(ke / 2) : 1.f;
  const float s2 = mul_scale ? pow2f_exact(ke - ke / 2) : 1.f;
  const int NY = g.ny;
  const float rNX = 1.f / static_cast<float>(NX), rNXY = 1.f / static_cast<float>(NXY);
  const bool pairs = (reinterpret_cast<uintptr_t>(f) & 15u) == 0;
  auto load_f = [&](int base, double (&v)[kCdfPer]) {
    const int l0 = base + static_cast<int>(threadIdx.x) * kCdfPer;
    if (pairs && l0 + kCdfPer <= nv) {
#pragma unroll
      for (int r = 0; r < kCdfPer; r += 2) {
        const double2 q = __ldg(reinterpret_cast<const double2*>(f + l0 + r));
        v[r] = q.x;
        v[r + 1] = q.y;
      }
    } else {
#pragma unroll
      for (int r = 0; r < kCdfPer; ++r) v[r] = (l0 + r < nv) ? __ldg(f + l0 + r) : 0.0;
    }
  };
  double fv[kCdfPer];
  load_f(0, fv);
  long long carry_e = 0, carry_d = 0;
  for (int base = 0; base < nv; base += kCdfChunk) {
    double fn[kCdfPer];
    if (base + kCdfChunk < nv) load_f(base + kCdfChunk, fn);
    const int l0 = base + static_cast<int>(threadIdx.x) * kCdfPer;
    int ii = 0, jj = 0, kk = 0;
    if (vr && l0 < nv) node_ijk(l0, NX, NXY, rNX, rNXY, ii, jj, kk);
    long long pe[kCdfPer], ad[kCdfPer];
    int sgn = 0;  // bit r: the sign of node l0 + r
#pragma unroll
    for (int r = 0; r < kCdfPer; ++r) {
      const int l = l0 + r;
      long long te = 0, td = 0;
      if (l < nv) {
        const long long F = to_fixed_s(fv[r], kc, bad);
        if (vr) {
          const dfl ev = dfl_mul(dfl_mul(s_fac[ii], s_fac[kMaxAxis + jj]),
                                 s_fac[2 * kMaxAxis + kk]);
          const long long E =
              mul_scale ? to_fixed_f_mul(ev.hi, s1, s2, bad) + to_fixed_f_mul(ev.lo, s1, s2, bad)
                        : to_fixed_f(ev.hi, ke, bad) + to_fixed_f(ev.lo, ke, bad);
          if (recompute) te = E;
          const long long d = F - E;
          sgn |= (d < 0 ? 1 : 0) << r;
          td = d < 0 ? -d : d;
          if (++ii == NX) { ii = 0; if (++jj == NY) { jj = 0; ++kk; } }
        } else {
          sgn |= static_cast<int>(static_cast<unsigned long long>(__double_as_longlong(fv[r])) >> 63) << r;
          td = F < 0 ? -F : F;
        }
      }
      pe[r] = te + (r ? pe[r - 1] : 0);
      ad[r] = td + (r ? ad[r - 1] : 0);
    }
    // the scan's shared words are rewritten by the next chunk only after every thread has
    // passed this chunk's second barrier, i.e. read its totals
    long long oe = pe[kCdfPer - 1], od = ad[kCdfPer - 1], te, td;
    block_scan2_i64(oe, od, te, td, &s_scan[0][0]);
    oe += carry_e;
    od += carry_d;
    // the cumulative sums at positions p = node + 1 as 2 c + s (s = 1: the node is negative,
    // the sign that picks the sign of a partner's contribution), through the warp's
    // transpose, and the coarse index
#pragma unroll
    for (int r = 0; r < kCdfPer; ++r) {
      tr_e[lane * kCdfPitch + r] = (oe + pe[r]) << 1;
      tr_d[lane * kCdfPitch + r] = ((od + ad[r]) << 1) | ((sgn >> r) & 1);
    }
    __syncwarp();
    const int wbase = base + warp * 32 * kCdfPer;
#pragma unroll
    for (int r = 0; r < kCdfPer; ++r) {
      const int v = r * 32 + lane;
      const int p = wbase + v + 1;
      if (p <= nv) {
        const int idx = (v / kCdfPer) * kCdfPitch + v % kCdfPer;
        const long long ve = tr_e[idx], vd = tr_d[idx];
        if (recompute) ce[p] = ve;
        cd[p] = vd;
        if ((p & (cstep - 1)) == 0) {
          s_coarse[0][p / cstep] = ve >> 1;
          s_coarse[1][p / cstep] = vd >> 1;
        }
      }
    }
    __syncwarp();  // the transpose is rewritten by the next chunk
    carry_e += te;
    carry_d += td;
#pragma unroll
    for (int r = 0; r < kCdfPer; ++r) fv[r] = fn[r];
  }
  if (threadIdx.x == 0) {
    if (recompute) ce[0] = 0;
    cd[0] = 0;
    s_coarse[0][0] = 0;
    s_coarse[1][0] = 0;
    // the scale did not hold: a sum at or above 2^62 leaves no room for the sign bit
    if (carry_e < 0 || carry_d < 0 || carry_e >= (1ll << 62) || carry_d >= (1ll << 62))
      bad |= DVM_EW_NONFINITE;
  }
  __syncthreads();

  // Bucket tables, variance_reduction.f90:471-493: right(r) is the first l >= 1 with
  // cum(l) >= target(r), target(r) = floor(r T / 1000) with T = cum(n) (the reference's
  // r * 0.001 * cum(n), here exact); left(r) = right(r-1) - 1; right(1000) = n. The coarse
  // index narrows each lookup to cstep entries.
  const int ntab = vr ? 2 : 1;
  for (int t = 0; t < ntab; ++t) {
    if (vr && t == 0 && !recompute) continue;  // cached equilibrium: table unchanged
    const int ti = (vr && t == 0) ? 0 : 1;
    const long long* cum = (ti == 0) ? ce : cd;
    const long long tot = (ti == 0) ? carry_e : carry_d;
    const long long Tq = tot / 1000, Tr = tot % 1000;
    // a thread's targets (up to kPer) are searched in lockstep: the coarse index in shared
    // memory first, then the fine searches in global memory advance together, so their
    // dependent loads overlap instead of following one another
    constexpr int kPer = (kNRef + kCdfThreads - 1) / kCdfThreads;
    long long tg[kPer];
    int plo[kPer], phi[kPer];
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int r = threadIdx.x + 1 + j * kCdfThreads;
      plo[j] = 1;
      phi[j] = 1;  // empty: nothing to search
      tg[j] = 0;
      if (r <= kNRef) {
        const long long target = Tq * r + (Tr * r) / 1000;
        tg[j] = target;
        int lo = 0, hi = ncoarse + 1;  // first coarse entry >= target
        while (lo < hi) {
          const int mid = (lo + hi) >> 1;
          if (target > s_coarse[ti][mid]) lo = mid + 1; else hi = mid;
        }
        int pl = (lo == 0) ? 1 : (lo - 1) * cstep + 1;
        int ph = (lo > ncoarse) ? nv : lo * cstep;
        if (pl < 1) pl = 1;
        plo[j] = pl;
        phi[j] = ph > nv ? nv : ph;
      }
    }
    for (int it = 0; it < 64; ++it) {  // first p in [plo, phi] with cum(p) >= target
      bool open = false;
#pragma unroll
      for (int j = 0; j < kPer; ++j) {
        if (plo[j] < phi[j]) {
          open = true;
          const int mid = (plo[j] + phi[j]) >> 1;
          if (tg[j] > (cum[mid] >> 1)) plo[j] = mid + 1; else phi[j] = mid;
        }
      }
      if (!open) break;
    }
#pragma unroll
    for (int j = 0; j < kPer; ++j) {
      const int r = threadIdx.x + 1 + j * kCdfThreads;
      if (r <= kNRef) s_right[t][r - 1] = plo[j];
    }
  }
  __syncthreads();
  for (int t = 0; t < ntab; ++t) {
    if (vr && t == 0 && !recompute) continue;
    int2* ref = ((vr && t == 0) ? a.ref_eq : a.ref_dev) + static_cast<size_t>(cell) * kNRef;
    for (int r = threadIdx.x + 1; r <= kNRef; r += kCdfThreads) {
      int2 e;
      e.x = (r == 1) ? 0 : s_right[t][r - 2] - 1;
      e.y = (r == kNRef) ? nv : s_right[t][r - 1];
      ref[r - 1] = e;
    }
  }
  if (bad) atomicOr(a.err, bad);

  // Sample plan of this cell-step.
  if (threadIdx.x == 0) {
    CellPlan pl;
    const CollParams& cp = a.cp;
    const double qk = ldexp(1.0, -k);
    if (vr) {
      const double dens = P[DVM_P_DENS], temp = P[DVM_P_SPECIES_TEMP];
      const long long te = recompute ? carry_e : (ce[nv] >> 1);
      const double eq_dens = static_cast<double>(te) * ldexp(1.0, -ke);
      const double neq_dens = static_cast<double>(carry_d) * ldexp(1.0, -ke);
      const double fc = cp.dt * 0.5 / cp.Kn;  // n = m: factor_coeff = dt*0.5/Kn
      const double r = 0.5 * neq_dens / dens;
      const double dA[3] = {1.0, r, r}, dB[3] = {r, 1.0, r};
      const double nA[3] = {eq_dens, neq_dens, neq_dens}, nB[3] = {neq_dens, eq_dens, neq_dens};
      if (a.pairs.active) {
        for (int q = 0; q < 3; ++q) pl.num[q] = a.pairs.count[q];
      } else if (cp.samples_mode == DVM_SAMPLES_FIXED) {
        double w[3] = {dA[0] * dB[0], dA[1] * dB[1], dA[2] * dB[2]};
        if (!(dens > 0.0)) w[0] = w[1] = w[2] = 0.0;
        // in proportion to densA*densB, the last sub-integral taking the remainder so the
        // counts add up to samples_per_step
        const double W = w[0] + w[1] + w[2];
        const long long S = cp.samples_per_step;
        long long used = 0;
        for (int q = 0; q < 3; ++q) {
          long long nq = 0;
          if (W > 0.0) {
            if (q == 2) nq = (S - used) > 0 ? (S - used) : 0;
            else nq = llround(static_cast<double>(S) * (w[q] / W));
            if (nq > S - used) nq = S - used;
          }
          pl.num[q] = nq;
          used += nq;
        }
      } else {
        const double ct = pow(0.5 * (temp + temp), 2.0 / 3.0);
        for (int q = 0; q < 3; ++q)
          pl.num[q] = (dens > 0.0) ? num_coll_pairs(cp, ct, dA[q], dB[q]) : 0;
      }
      for (int q = 0; q < 3; ++q)
        pl.factor[q] = (pl.num[q] > 0)
                           ? fc * cp.sigma * nA[q] * nB[q] / static_cast<double>(pl.num[q])
                           : 0.0;
    } else {
      const double dens = P[DVM_P_DENS], temp = P[DVM_P_TEMP];
      const double neg = 0.5 * (dens - static_cast<double>(carry_d) * qk);
      const double absd = dens - 2.0 * neg;
      long long num;
      if (a.pairs.active) num = a.pairs.count[0];
      else if (cp.samples_mode == DVM_SAMPLES_FIXED) num = (dens > 0.0) ? cp.samples_per_step : 0;
      else num = (dens > 0.0) ? num_coll_pairs(cp, pow(0.5 * (temp + temp), 2.0 / 3.0),
                                               absd / dens, absd / dens) : 0;
      double factor = (num > 0) ? (cp.dt / cp.Kn) * cp.sigma * absd * absd / static_cast<double>(num)
                                : 0.0;
      factor = 0.5 * factor;
      pl.num[0] = num; pl.num[1] = 0; pl.num[2] = 0;
      pl.factor[0] = factor; pl.factor[1] = 0.0; pl.factor[2] = 0.0;
    }
    a.plan[cell] = pl;
  }
}

template <int T>
__global__ void __launch_bounds__(T, 1024 / T) k_cdf(CdfArgs a) {
  cdf_cta<T>(a, blockIdx.x);
}

template <int T>
static cudaError_t launch_cdf_t(const CdfArgs& a, cudaStream_t s) {
  constexpr int smem = (T / 32) * kCdfTrWarp * static_cast<int>(sizeof(long long));
  const cudaError_t e = cudaFuncSetAttribute(k_cdf<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_cdf<T><<<a.ncells, T, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_cdf(const CdfArgs& a, cudaStream_t s) {
  // one CTA per cell: as wide as still lets every cell's CTA be resident at once (1024
  // threads, one per SM; 512, two; otherwise 256, four)
  const int nsm = sm_count();
  if (a.ncells <= nsm) return launch_cdf_t<1024>(a, s);
  if (a.ncells <= 2 * nsm) return launch_cdf_t<512>(a, s);
  return launch_cdf_t<256>(a, s);
}

// ----------------------------------------------------------------------------------------
// k_plan: chunk offsets of every (cell, sub-integral) for the persistent collide kernel.
__device__ __forceinline__ void plan_cta(int ncells, const CellPlan* plan, long long* chunk_off,
                                         long long* total_samples, long long warps) {
  __shared__ long long s_w[32];
  __shared__ long long s_carry, s_samples, s_chunks;
  const int n = 3 * ncells;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) { s_carry = 0; s_samples = 0; s_chunks = 0; }
  __syncthreads();
  // the run length: as many chunks per run as leave every warp of the collide launch about
  // kRunsPerWarp runs (at least 1 chunk, at most kRunChunks)
  {
    long long c = 0;
    for (int e = threadIdx.x; e < n; e += blockDim.x)
      c += (plan[e / 3].num[e % 3] + kChunkSamples - 1) / kChunkSamples;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0 && c > 0)
      atomicAdd(reinterpret_cast<unsigned long long*>(&s_chunks), static_cast<unsigned long long>(c));
  }
  __syncthreads();
  const long long want = (warps > 0 ? warps : 1) * kRunsPerWarp;
  const long long runlen = max(1ll, min(static_cast<long long>(kRunChunks), s_chunks / want));
  for (int base = 0; base < n; base += 1024) {
    const int e = base + threadIdx.x;
    long long num = 0;
    if (e < n) num = plan[e / 3].num[e % 3];
    long long ch = (num + kChunkSamples * runlen - 1) / (kChunkSamples * runlen);
    long long v = ch;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const long long t = __shfl_up_sync(0xffffffffu, v, o);
      if (lane >= o) v += t;
    }
    if (lane == 31) s_w[warp] = v;
    __syncthreads();
    if (warp == 0) {
      long long w = s_w[lane];
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const long long t = __shfl_up_sync(0xffffffffu, w, o);
        if (lane >= o) w += t;
      }
      s_w[lane] = w;
    }
    __syncthreads();
    const long long incl = v + (warp > 0 ? s_w[warp - 1] : 0) + s_carry;
    if (e < n) chunk_off[e] = incl - ch;
    long long wsum = num;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) wsum += __shfl_xor_sync(0xffffffffu, wsum, o);
    if (lane == 0 && wsum > 0)
      atomicAdd(reinterpret_cast<unsigned long long*>(&s_samples),
                static_cast<unsigned long long>(wsum));
    __syncthreads();
    if (threadIdx.x == 0) s_carry += s_w[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    chunk_off[n] = s_carry | (runlen << kRunShift);
    *total_samples = s_samples;
  }
}

__global__ void __launch_bounds__(1024) k_plan(int ncells, const CellPlan* plan,
                                               long long* chunk_off, long long* total_samples,
                                               long long warps) {
  plan_cta(ncells, plan, chunk_off, total_samples, warps);
}

cudaError_t launch_plan(int ncells, const CellPlan* plan, long long* chunk_off,
                        long long* total_samples, long long warps, cudaStream_t s) {
  k_plan<<<1, 1024, 0, s>>>(ncells, plan, chunk_off, total_samples, warps);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// k_collide: persistent; a chunk is kChunkSamples consecutive samples of one
// (cell, sub-integral). One thread per sample.
//
// GB300 runs FP64 at 1/64 of its FP32 rate, so this kernel moves its arithmetic off the
// FP64 pipe: the partner search compares exact fixed-point integers (the CDFs of k_cdf and
// the target floor(R T) formed from the 53-bit integer behind R), the remap uses tables of
// node differences / reciprocals / denominator terms, a table of g and g^(2-2 omega) on
// cubic uniform grids, the exact 1/2 mass ratios of like-species pairs, and hi + lo float
// pairs for the post-collision velocities, the remap weights and the contributions. Each
// of these changes a value by at most about 2^-46 relative; the parity bar (1e-12 of
// max|f| against the restatement) checks the sum.

// R 2^53 truncated, from the bits of R in [0, 1): the 53-bit integer behind a Philox
// uniform, exactly.
__device__ __forceinline__ unsigned long long u53_bits(double R) {
  const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(R));
  const int e = static_cast<int>((b >> 52) & 0x7ff);
  if (e == 0 || e > 1022 || 1022 - e >= 64) return 0;
  return ((b & ((1ull << 52) - 1)) | (1ull << 52)) >> (1022 - e);
}

// referenced_search (utils/sort_and_search.f90:40-86) on the fixed-point CDF: bucket
// ceil(1000 R), then the index idx with cum(idx) < R cum(n) <= cum(idx+1), the target
// floor(R T) and the bucket index formed exactly in integers. The buckets of k_cdf are
// built with the same exact targets, so the answer always lies inside its bucket, and it
// is unique (the last index whose cumulative value is below the target), so any exact
// search returns the reference's bisection answer. Here the bucket is narrowed four ways
// per step (three independent loads), which takes about half the dependent load rounds
// of bisection on the wide tail buckets that set a warp's pace. The reference's test
// cum(idx) < target <= cum(idx+1) is made on the bucket's ends instead, loaded beside the
// first round: every step keeps cum(lo) < target <= cum(hi) and the sums never decrease,
// so the test on the ends holds exactly when it holds on the result. The stored values
// are 2 cum + s (s the sign bit of k_cdf); against the doubled target every comparison
// has the outcome it has on cum itself, so the sign bits change no step.
// R enters as m = R 2^53 truncated and the test R < tol, made by the caller (on m for the
// Philox uniforms, on the double for recorded ones).
__device__ __forceinline__ int referenced_search_fixed(const long long* __restrict__ cum,
                                                       const int2* __restrict__ ref, int n,
                                                       unsigned long long m, bool below_tol,
                                                       uint32_t& bad) {
  if (below_tol) return 0;  // R < tol
  int i = static_cast<int>((1000ull * m + ((1ull << 53) - 1)) >> 53);
  i = i < 1 ? 1 : (i > kNRef ? kNRef : i);
  const int2 lr = __ldg(ref + i - 1);
  const int left = lr.x, right = lr.y;
  if (left == right) return left < n ? left : n - 1;
  const unsigned long long T = static_cast<unsigned long long>(__ldg(cum + n) >> 1);
  // the target floor(R T), doubled: 2 t > 2 c + s exactly when t > c (s = 0 or 1)
  const long long adj =
      static_cast<long long>((__umul64hi(m, T) << 11) | ((m * T) >> 53)) << 1;
  // cum(lo) < adj <= cum(hi) holds for a valid bucket; each step keeps it
  int lo = left, hi = right;
  if (lo >= 0 && hi <= n && lo < hi) {
    const long long c_lo = __ldg(cum + lo), c_hi = __ldg(cum + hi);
    for (int it = 0; hi - lo > 1 && it < kMaxSearchIters; ++it) {
      const int span = hi - lo;
      int nlo = lo, nhi = hi;
#pragma unroll
      for (int j = 1; j < 4; ++j) {
        const int p = lo + ((span * j) >> 2);
        if (adj > __ldg(cum + p)) nlo = max(nlo, p); else nhi = min(nhi, p);
      }
      lo = nlo;
      hi = nhi;
    }
    if (hi - lo == 1 && lo < n && adj > c_lo && adj <= c_hi) return lo;
  }
  bad |= DVM_EW_SEARCH;
  int blo = 0, bhi = n;
  while (bhi - blo > 1) {
    const int mid = blo + (bhi - blo) / 2;
    if (adj > __ldg(cum + mid)) blo = mid; else bhi = mid;
  }
  return blo;
}

// ---- the FP64 collide arithmetic on the FP32 pipe ---------------------------------------
// Post-collision velocities, remap weights and contributions are formed in hi + lo float
// pairs (dfloat.cuh, about 47 significant bits); the few steps whose outcome the reference's
// FP64 rounding decides stay in FP64: the bucket choice ceil(1000 R) and the search target
// R * cum(n) of each partner pick. The contributions go to the FP64 atomics as doubles.
__device__ __forceinline__ int okeyf(float d);

struct AxisEntryD {
  dfl D[kTabW];
  dfl invD[kTabW];
  dfl T[kTabW];
};

struct SmemAxesD {
  const double* vd[3];      // FP64 nodes (the rare boundary-stencil path)
  const dfl* v[3];          // nodes as pairs
  const long long* mid[3];  // pair keys of the midpoints between consecutive nodes
  const AxisEntryD* tab[3];
  int n[3];
};

// Order-preserving key of a normalised pair (|lo| at most half an ulp of hi).
__device__ __forceinline__ long long dkey(dfl a) {
  const uint32_t h = static_cast<uint32_t>(okeyf(a.hi));
  const uint32_t l = static_cast<uint32_t>(okeyf(a.lo)) ^ 0x80000000u;
  return static_cast<long long>((static_cast<uint64_t>(h) << 32) | l);
}

__device__ __forceinline__ int dfl_isgn(dfl a) {
  return (a.hi < 0.f || (a.hi == 0.f && a.lo < 0.f)) ? -1 : 1;
}

// Nearest integer (ties to even) of x, as __float2int_rn for |x| <= 2^22, by the FP32 adder:
// x + 1.5 2^23 lies in [2^23, 2^24], where the float spacing is 1 and the even offset keeps
// the parity of the tie rule. Larger |x| (and NaN) are clamped to +-2^22 first; the callers
// clamp the result to an axis much shorter than that.
__device__ __forceinline__ int round_small(float x) {
  x = fminf(fmaxf(x, -4194304.f), 4194304.f);
  return __float_as_int(__fadd_rn(x, 12582912.f)) - 0x4B400000;
}

// Nearest node, as nearest() but on pair keys.
// kUniform (a uniform axis): x = factor (u.hi - vmin) is u's position in node units up to
// a few FP32 roundings (of u.hi - vmin, of the factor, of the product) and the dropped
// u.lo, each relative to values below about 4 n in node units: under 2e-4 for the longest
// axis (128 nodes). When x lies within 0.499 of the node it rounds to, no midpoint is
// nearer and the exact check is skipped; a position clamped to an end node is that node.
// The other positions (0.2 % of them) are checked on the keys as on any axis.
template <bool kUniform>
__device__ __forceinline__ int nearest_d(const SmemAxesD& A, int ax, dfl u, float vmin,
                                         float factor, int& corner, int& bad) {
  const int mx = A.n[ax] - 1;
  const float x = factor * (u.hi - vmin);
  int o = round_small(x);
  const bool check = !kUniform || !(fabsf(x - static_cast<float>(o)) < 0.499f);
  o = o < 0 ? 0 : (o > mx ? mx : o);
  if (u.hi != u.hi) bad |= 1;
  if (check) {
    const long long* mid = A.mid[ax];
    const long long vk = dkey(u);
    int it = 0;
    while (o > 0 && vk <= mid[o - 1] && it++ < kMaxAxis) --o;
    while (o < mx && vk > mid[o] && it++ < kMaxAxis) ++o;
  }
  if (o >= mx) { o = mx; corner++; }
  else if (o <= 0) { o = 0; corner++; }
  return o;
}

// Per-axis terms of the remap, in two parts so that each is loaded when it is needed:
// the interior difference and the denominator term (for f_e), then the reciprocal of the
// interior difference and the exterior difference (for the axis weight).
__device__ __forceinline__ void axis_den(const SmemAxesD& A, int ax, int o, int s, int avail,
                                         dfl& int_d, dfl& t_d) {
  t_d = dfl_make(0.f, 0.f);
  if (s >= -kTabS && s <= kTabS) {
    const AxisEntryD& e = A.tab[ax][o];
    int_d = e.D[kTabS + s];
    if (avail) t_d = e.T[kTabS + s];
  } else {
    const dfl* v = A.v[ax];
    int_d = dfl_sub(v[o + s], v[o]);
    if (avail) {
      const dfl ext_d = dfl_sub(v[o - s], v[o]);
      t_d = dfl_mul(ext_d, dfl_sub(ext_d, int_d));
    }
  }
}

__device__ __forceinline__ void axis_ext(const SmemAxesD& A, int ax, int o, int s, int avail,
                                         dfl& inv_d, dfl& ext_d) {
  ext_d = dfl_make(0.f, 0.f);
  if (s >= -kTabS && s <= kTabS) {
    const AxisEntryD& e = A.tab[ax][o];
    inv_d = e.invD[kTabS + s];
    if (avail) ext_d = e.D[kTabS - s];
  } else {
    const dfl* v = A.v[ax];
    inv_d = dfl_div(dfl_make(1.f, 0.f), dfl_sub(v[o + s], v[o]));
    if (avail) ext_d = dfl_sub(v[o - s], v[o]);
  }
}

// compute_remapping_quantities (collisions/remapping.f90:92-394), f_off = 1, in pairs,
// with the replenishment scatter of the contribution w8 (apply_phi_replenishment,
// replenishing_collisions.f90:356-434) into f.
template <bool kUniform>
__device__ __forceinline__ int remap_scatter_dfl(const GridInfo& g, const SmemAxesD& A, dfl u,
                                                 dfl v, dfl w, float xmin, float ymin,
                                                 float zmin, float xfac, float yfac, float zfac,
                                                 double* f, dfl w8, uint32_t& nat) {
  int corner = 0, bad = 0;
  int o_i = nearest_d<kUniform>(A, 0, u, xmin, xfac, corner, bad);
  int o_j = nearest_d<kUniform>(A, 1, v, ymin, yfac, corner, bad);
  int o_k = nearest_d<kUniform>(A, 2, w, zmin, zfac, corner, bad);
  const int i_max = g.nx - 1, j_max = g.ny - 1, k_max = g.nz - 1;
  if (corner == 3) {
    o_i -= isign1(o_i - 1);
    o_j -= isign1(o_j - 1);
    o_k -= isign1(o_k - 1);
  }
  const dfl a = dfl_sub(u, A.v[0][o_i]), b = dfl_sub(v, A.v[1][o_j]), c = dfl_sub(w, A.v[2][o_k]);
  int sa = dfl_isgn(a), sb = dfl_isgn(b), sc = dfl_isgn(c);
  if (o_i + sa > i_max || o_i + sa < 0) {
    sa = -1 * sa;
    find_boundary_stencil(sa, sb, sc, dfl_to_double(a), o_i, o_j, o_k, A.vd[0], A.vd[1], A.vd[2],
                          0, i_max, 0, j_max, 0, k_max);
  }
  if (o_j + sb > j_max || o_j + sb < 0) {
    sb = -1 * sb;
    find_boundary_stencil(sb, sa, sc, dfl_to_double(b), o_j, o_i, o_k, A.vd[1], A.vd[0], A.vd[2],
                          0, j_max, 0, i_max, 0, k_max);
  }
  if (o_k + sc > k_max || o_k + sc < 0) {
    sc = -1 * sc;
    find_boundary_stencil(sc, sb, sa, dfl_to_double(c), o_k, o_j, o_i, A.vd[2], A.vd[1], A.vd[0],
                          0, k_max, 0, j_max, 0, i_max);
  }
  const int fx = (o_i - sa <= i_max && o_i - sa >= 0);
  const int fy = (o_j - sb <= j_max && o_j - sb >= 0);
  const int fz = (o_k - sc <= k_max && o_k - sc >= 0);
  const dfl zero = dfl_make(0.f, 0.f);
  dfl f_e = zero;
  if (!(fx | fy | fz)) {
    bad |= 2;
  } else {
    dfl int_x, t_x, int_y, t_y, int_z, t_z;
    axis_den(A, 0, o_i, sa, fx, int_x, t_x);
    axis_den(A, 1, o_j, sb, fy, int_y, t_y);
    axis_den(A, 2, o_k, sc, fz, int_z, t_z);
    // (a^2 + b^2 + c^2 - a int_x - b int_y - c int_z) / den, den = the available T terms
    const dfl num = dfl_add(dfl_add(dfl_mul(a, dfl_sub(a, int_x)), dfl_mul(b, dfl_sub(b, int_y))),
                            dfl_mul(c, dfl_sub(c, int_z)));
    dfl den = fx ? t_x : zero;
    if (fy) den = dfl_add(den, t_y);
    if (fz) den = dfl_add(den, t_z);
    f_e = dfl_div(num, den);
  }
  if (bad & 2) return bad;
  nat += 4u + static_cast<uint32_t>(fx + fy + fz);
  // weights and their contributions w * mass, scattered as they are formed (the centre
  // node takes 1 - the others, as in the reference)
  const int NX = g.nx, NXY = g.nx * g.ny;
  const int base = o_i + NX * o_j + NXY * o_k;
  const double c_e = dfl_mul_to_double(w8, f_e);  // the exterior nodes' share
  if (fx) atomicAdd(f + base - sa, c_e);
  if (fy) atomicAdd(f + base - NX * sb, c_e);
  if (fz) atomicAdd(f + base - NXY * sc, c_e);
  // the weights' running sum starts from (number of exterior nodes) x f_e, the doubling
  // exact
  const int ne = fx + fy + fz;
  dfl sum = f_e;
  if (ne >= 2) sum = dfl_scale(f_e, 2.f);
  if (ne == 3) sum = dfl_add(sum, f_e);
  {
    dfl inv_x, ext_x;
    axis_ext(A, 0, o_i, sa, fx, inv_x, ext_x);
    const dfl f_ix = dfl_mul(dfl_sub(a, fx ? dfl_mul(f_e, ext_x) : zero), inv_x);
    atomicAdd(f + base + sa, dfl_mul_to_double(w8, f_ix));
    sum = dfl_add(sum, f_ix);
  }
  {
    dfl inv_y, ext_y;
    axis_ext(A, 1, o_j, sb, fy, inv_y, ext_y);
    const dfl f_iy = dfl_mul(dfl_sub(b, fy ? dfl_mul(f_e, ext_y) : zero), inv_y);
    atomicAdd(f + base + NX * sb, dfl_mul_to_double(w8, f_iy));
    sum = dfl_add(sum, f_iy);
  }
  {
    dfl inv_z, ext_z;
    axis_ext(A, 2, o_k, sc, fz, inv_z, ext_z);
    const dfl f_iz = dfl_mul(dfl_sub(c, fz ? dfl_mul(f_e, ext_z) : zero), inv_z);
    atomicAdd(f + base + NXY * sc, dfl_mul_to_double(w8, f_iz));
    sum = dfl_add(sum, f_iz);
  }
  const dfl f_o = dfl_sub(dfl_make(1.f, 0.f), sum);
  atomicAdd(f + base, dfl_mul_to_double(w8, f_o));
  return bad;
}

// Adds a warp's scatter counts to the launch total (every thread of the block calls it).
__device__ __forceinline__ void add_scatter_count(unsigned long long* total, uint32_t n) {
  if (!total) return;
  unsigned long long v = n;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if ((threadIdx.x & 31) == 0 && v) atomicAdd(total, v);
}

// t = R - k/kTrigN (k = the top 10 bits of R) as a pair, and k, from m = R 2^53 truncated.
__device__ __forceinline__ dfl angle_fraction(unsigned long long m, int& k) {
  k = static_cast<int>(m >> 43);
  const unsigned long long t = m & ((1ull << 43) - 1);
  const uint32_t th = static_cast<uint32_t>(t >> 20), tl = static_cast<uint32_t>(t & 0xfffffu);
  // exact floats of the 23- and 20-bit integers: (2^23 + n) - 2^23
  const float fh = __fsub_rn(__int_as_float(static_cast<int>(0x4B000000u | th)), 8388608.f);
  const float fl = __fsub_rn(__int_as_float(static_cast<int>(0x4B000000u | tl)), 8388608.f);
  return dfl_norm(fh * 0x1.0p-33f, fl * 0x1.0p-53f);
}

// Visiting order of the sample chunks: chunk(pos) = pos P mod total, a bijection of
// 0..total-1 for a prime P that does not divide total. A warp's positions advance by a fixed
// stride, so its chunks follow a running sum mod total: one 64-bit remainder per thread at
// the start instead of one per chunk.
struct ChunkWalk {
  unsigned long long cur = 0, step = 0;
  __device__ ChunkWalk(long long pos0, long long stride, long long tot) {
    if (tot <= 0) return;
    const unsigned long long total = static_cast<unsigned long long>(tot);
    const unsigned long long P = (total % 2147483647ull == 0) ? 2147483629ull : 2147483647ull;
    const unsigned __int128 pm = P % total;
    cur = static_cast<unsigned long long>(
        (static_cast<unsigned __int128>(static_cast<unsigned long long>(pos0) % total) * pm) % total);
    step = static_cast<unsigned long long>(
        (static_cast<unsigned __int128>(static_cast<unsigned long long>(stride) % total) * pm) % total);
  }
  __device__ __forceinline__ long long next(long long tot) {
    const unsigned long long c = cur;
    cur += step;
    if (cur >= static_cast<unsigned long long>(tot)) cur -= static_cast<unsigned long long>(tot);
    return static_cast<long long>(c);
  }
};

struct CollideSmem {
  size_t axes, axes_d, keys, tabs, gtab, trig, exp2tab, total;
};

__host__ __device__ inline CollideSmem collide_smem_layout(const GridInfo& g, const CollTables& t) {
  CollideSmem L;
  const size_t nsum = static_cast<size_t>(g.nx + g.ny + g.nz);
  L.axes = 0;
  L.axes_d = L.axes + nsum * sizeof(double);
  L.keys = L.axes_d + nsum * sizeof(dfl);
  L.tabs = L.keys + nsum * sizeof(long long);
  L.gtab = L.tabs + 3 * static_cast<size_t>(t.nmax) * sizeof(AxisEntryD);
  L.gtab = (L.gtab + 15) & ~static_cast<size_t>(15);  // double2 needs 16-byte alignment
  L.trig = L.gtab + (t.gtab_smem ? static_cast<size_t>(t.gtab_n) * sizeof(double2) : 0);
  L.exp2tab = L.trig + static_cast<size_t>(kTrigN) * sizeof(float4);
  // for the general kernel's powers: 2^(j/32), then the exponents (2 - 2 omega)/2 and
  // 1/alpha as three floats each (two float2 slots each)
  L.total = L.exp2tab + static_cast<size_t>(kExp2TabN + 4) * sizeof(float2);
  return L;
}

// The common configuration: Philox uniforms (no recorded list), one replica, isotropic
// scattering (alpha = 1) and the tabulated relative speeds of a cubic uniform grid. The
// collide kernels are also compiled for it alone (kFast): without the other branches they
// hold fewer registers live (the FP64 kernel's copy spills 24 bytes per thread, the general
// kernel 116).
static bool collide_fast(const CollideArgs& a) {
  return !a.pairs.active && a.cp.num_repl == 1 && a.t.gtab != nullptr &&
         !(fabs(1.0 / (0.5 * (a.cp.alpha + a.cp.alpha)) - 1.0) > kDoubleTol);
}

// The two 53-bit Philox integers of a sample's counter: from the key schedule in the
// launch parameters (kKeys; the single-context kernels, where each key is an operand) or
// from the seed (the grouped kernels, whose per-group parameters are read by index);
// kCall: through the out-of-line copy of the rounds.
template <bool kKeys, bool kCall = false>
__device__ __forceinline__ void sample_u53x2(const CollideArgs& a, uint32_t i, uint32_t cell,
                                             uint32_t step, uint32_t q, uint32_t call,
                                             unsigned long long& m0, unsigned long long& m1) {
  if (kKeys && kCall) philox_u53x2_rk_call(a.rk, i, cell, step, q, call, m0, m1);
  else if (kKeys) philox_u53x2_rk(a.rk, i, cell, step, q, call, m0, m1);
  else philox_u53x2(a.cp.seed, i, cell, step, q, call, m0, m1);
}

// One CTA of the persistent collide launch: CTA bid of the nblk that walk this grid's
// chunks; kFast: the configuration of collide_fast; kKeys: as sample_u53x2.
template <bool kFast, bool kKeys>
__device__ __forceinline__ void collide_cta(const CollideArgs& a, int bid, int nblk) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  const GridInfo& g = a.g;
  const CollideSmem L = collide_smem_layout(g, a.t);
  double* sv = reinterpret_cast<double*>(s_raw + L.axes);
  dfl* svd = reinterpret_cast<dfl*>(s_raw + L.axes_d);
  long long* sk = reinterpret_cast<long long*>(s_raw + L.keys);
  AxisEntryD* st = reinterpret_cast<AxisEntryD*>(s_raw + L.tabs);
  double2* sg = reinterpret_cast<double2*>(s_raw + L.gtab);
  float4* strig = reinterpret_cast<float4*>(s_raw + L.trig);
  const int nsum = g.nx + g.ny + g.nz;
  for (int t = threadIdx.x; t < nsum; t += blockDim.x) {
    const double* ax = t < g.nx ? g.x : (t < g.nx + g.ny ? g.y : g.z);
    const int n = t < g.nx ? g.nx : (t < g.nx + g.ny ? g.ny : g.nz);
    const int i = t < g.nx ? t : (t < g.nx + g.ny ? t - g.nx : t - g.nx - g.ny);
    sv[t] = ax[i];
    const dfl xv = dfl_from_double(ax[i]);
    svd[t] = dfl_norm(xv.hi, xv.lo);
    if (i + 1 < n) {
      const dfl m = dfl_from_double(0.5 * (ax[i] + ax[i + 1]));
      sk[t] = dkey(dfl_norm(m.hi, m.lo));
    } else {
      sk[t] = 0x7FFFFFFFFFFFFFFFLL;
    }
  }
  {
    const double* src = reinterpret_cast<const double*>(a.t.axis);
    dfl* dst = reinterpret_cast<dfl*>(st);
    const int n = 3 * a.t.nmax * static_cast<int>(sizeof(AxisEntry) / sizeof(double));
    for (int t = threadIdx.x; t < n; t += blockDim.x) {
      const dfl v = dfl_from_double(src[t]);
      dst[t] = dfl_norm(v.hi, v.lo);
    }
  }
  if (a.t.gtab_smem)
    for (int t = threadIdx.x; t < a.t.gtab_n; t += blockDim.x) sg[t] = a.t.gtab[t];
  for (int t = threadIdx.x; t < kTrigN; t += blockDim.x) {
    const double2 cs = a.t.trig[t];
    const dfl c = dfl_from_double(cs.x), sn = dfl_from_double(cs.y);
    const dfl cn = dfl_norm(c.hi, c.lo), snn = dfl_norm(sn.hi, sn.lo);
    strig[t] = make_float4(cn.hi, cn.lo, snn.hi, snn.lo);
  }
  float2* sexp2 = reinterpret_cast<float2*>(s_raw + L.exp2tab);
  if (!kFast) {
    for (int t = threadIdx.x; t < kExp2TabN + 2; t += blockDim.x) {
      if (t < kExp2TabN) {
        sexp2[t] = exp2_table_entry(t);
      } else {
        const double e = (t == kExp2TabN)
                             ? 0.5 * (2.0 - 2.0 * (0.5 * (a.cp.omega + a.cp.omega)))
                             : 1.0 / (0.5 * (a.cp.alpha + a.cp.alpha));
        const flt3 q = flt3_from_double(e);
        const int o = kExp2TabN + 2 * (t - kExp2TabN);
        sexp2[o] = make_float2(q.hi, q.mid);
        sexp2[o + 1] = make_float2(q.lo, 0.f);
      }
    }
  }
  __syncthreads();
  SmemAxesD A;
  A.vd[0] = sv; A.vd[1] = sv + g.nx; A.vd[2] = sv + g.nx + g.ny;
  A.v[0] = svd; A.v[1] = svd + g.nx; A.v[2] = svd + g.nx + g.ny;
  A.mid[0] = sk; A.mid[1] = sk + g.nx; A.mid[2] = sk + g.nx + g.ny;
  A.tab[0] = st; A.tab[1] = st + a.t.nmax; A.tab[2] = st + 2 * a.t.nmax;
  A.n[0] = g.nx; A.n[1] = g.ny; A.n[2] = g.nz;
  const double2* gtab = a.t.gtab_smem ? sg : a.t.gtab;
  dfl two_pi;
  {
    const dfl t = dfl_from_double(a.t.two_pi);
    two_pi = dfl_norm(t.hi, t.lo);
  }
  const dfl one_sixth = dfl_make(0x1.555556p-3f, -0x1.555556p-28f);  // 1/6 to 2^-50

  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const int nent = 3 * a.ncells;
  const long long total = a.chunk_off[nent] & kRunMask;
  const int runlen = static_cast<int>(a.chunk_off[nent] >> kRunShift);
  const bool vr = (a.cp.method == DVM_COLL_VR);
  const int NR = kFast ? 1 : a.cp.num_repl;
  const double vhs = 2.0 - 2.0 * (0.5 * (a.cp.omega + a.cp.omega));
  const double alpha = 0.5 * (a.cp.alpha + a.cp.alpha);
  const double ralpha = 1.0 / alpha;
  const bool vss = kFast ? false : (fabs(ralpha - 1.0) > kDoubleTol);
  const uint32_t step = a.step_dev ? *a.step_dev : a.step;
  uint32_t bad = 0;
  uint32_t nat = 0;  // FP64 adds into f by this thread

  // one warp per chunk; chunks are visited in a scattered order (a bijection of
  // 0..total-1), so the warps in flight at any moment work on many cells and their FP64
  // atomics spread over many f slabs instead of piling onto the busiest nodes of one cell
  const int wpb = blockDim.x >> 5;
  const long long pos0 = static_cast<long long>(bid) * wpb + (threadIdx.x >> 5);
  const long long stride = static_cast<long long>(nblk) * wpb;
  ChunkWalk walk(pos0, stride, total);
  for (long long pos = pos0; pos < total; pos += stride) {
    const long long chunk = walk.next(total);
    int lo = 0, hi = nent;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (a.chunk_off[mid] <= chunk) lo = mid; else hi = mid;
    }
    const int cell = lo / 3, q = lo - 3 * (lo / 3);
    const CellPlan& pl = a.plan[cell];
    const double factor = pl.factor[q];
    const size_t cs = static_cast<size_t>(cell) * (nv + 1);
    double* f = a.f + static_cast<size_t>(cell) * nv;
    // the run's chunks of 32 samples, one after another
    const long long i0 =
        (chunk - a.chunk_off[lo]) * (kChunkSamples * runlen) + (threadIdx.x & 31);
    for (int rr = 0; rr < runlen; ++rr) {
    const long long i = i0 + rr * kChunkSamples;
    if (i >= pl.num[q]) break;

    // partners: pick_collision_partner x2 (collision_utilities.f90:142-186)
    unsigned long long mA = 0, mB = 0;
    const bool rec = kFast ? false : a.pairs.active;
    if (!rec) sample_u53x2<kKeys, true>(a, static_cast<uint32_t>(i), cell, step, q, 0u, mA, mB);
    int lA, lB;
    if (rec && a.pairs.glA[q]) {
      lA = a.pairs.glA[q][i];
      lB = a.pairs.glB[q][i];
    } else {
      bool tA = mA < kTolU53, tB = mB < kTolU53;
      if (rec) {
        const double rA = a.pairs.rA[q][i], rB = a.pairs.rB[q][i];
        mA = u53_bits(rA); mB = u53_bits(rB);
        tA = __double_as_longlong(rA) < __double_as_longlong(kDoubleTol);
        tB = __double_as_longlong(rB) < __double_as_longlong(kDoubleTol);
      }
      const bool aeq = vr && q == 0, beq = vr && q == 1;
      lA = referenced_search_fixed((aeq ? a.cum_eq : a.cum_dev) + cs,
                                  (aeq ? a.ref_eq : a.ref_dev) + static_cast<size_t>(cell) * kNRef,
                                  nv, mA, tA, bad);
      lB = referenced_search_fixed((beq ? a.cum_eq : a.cum_dev) + cs,
                                  (beq ? a.ref_eq : a.ref_dev) + static_cast<size_t>(cell) * kNRef,
                                  nv, mB, tB, bad);
    }
    int iA, jA, kA, iB, jB, kB;
    node_ijk(lA, NX, NXY, a.rnx, a.rnxy, iA, jA, kA);
    node_ijk(lB, NX, NXY, a.rnx, a.rnxy, iB, jB, kB);
    // compute_relative_velocity (collision_utilities.f90:188-218) and g^(2-2 omega)
    double gg, g_sigma;
    if (kFast || gtab) {
      const int di = iB - iA, dj = jB - jA, dk = kB - kA;
      const int s2 = di * di + dj * dj + dk * dk;
      if (s2 == 0) continue;  // g < double_tol, variance_reduction.f90:697
      const double2 e = gtab[s2];
      gg = e.x;
      g_sigma = e.y;
    } else {
      // |g|^2 from the nodes as pairs, |g| by the pair square root and g^(2 - 2 omega) as
      // (|g|^2)^((2 - 2 omega)/2) by dfl_pow: the FP64 sqrt and pow they replace took half
      // of the kernel's time on grids without a speed table
      const dfl gxp = dfl_sub(A.v[0][iB], A.v[0][iA]), gyp = dfl_sub(A.v[1][jB], A.v[1][jA]);
      const dfl gzp = dfl_sub(A.v[2][kB], A.v[2][kA]);
      const dfl g2 = dfl_add(dfl_add(dfl_mul(gxp, gxp), dfl_mul(gyp, gyp)), dfl_mul(gzp, gzp));
      const dfl gp = dfl_sqrt(g2);
      gg = dfl_to_double(gp);
      if (gg < kDoubleTol) continue;
      if (vhs == 1.0) {
        g_sigma = gg;
      } else {
        const float2 qa = sexp2[kExp2TabN], qb = sexp2[kExp2TabN + 1];
        flt3 q;
        q.hi = qa.x; q.mid = qa.y; q.lo = qb.x;
        g_sigma = dfl_to_double(dfl_pow(g2, q, sexp2));
      }
    }
    // signs of the deviation partners (cdf_neq%sign); FMC: sign of phi_old. The low bit of
    // the value closing the partner's interval, next to the last values the search read
    const bool negA =
        (vr && q == 0) ? false : (__ldg(a.cum_dev + cs + lA + 1) & 1) != 0;
    const bool negB =
        (vr && q == 1) ? false : (__ldg(a.cum_dev + cs + lB + 1) & 1) != 0;
    // vr_depletion_routine elastic part (variance_reduction.f90:1157-1166): kin_depl(1) =
    // kin_depl(2) = sA sB factor g^(2-2 omega)
    const double fg = factor * g_sigma;
    const double kin = (negA != negB) ? -fg : fg;
    atomicAdd(f + lA, -kin);
    atomicAdd(f + lB, -kin);
    nat += 2u;
    // replenish_collision elastic branch (replenishing_collisions.f90:206-249)
    dfl kr;
    {
      double kin_r = kin;
      if (NR != 1) kin_r = kin / static_cast<double>(NR);
      const dfl t = dfl_from_double(kin_r);
      kr = dfl_norm(t.hi, t.lo);
    }
    // v_com of a like-species pair: (xi_A + xi_B) / 2
    const dfl vc0 = dfl_scale(dfl_add(A.v[0][iA], A.v[0][iB]), 0.5f);
    const dfl vc1 = dfl_scale(dfl_add(A.v[1][jA], A.v[1][jB]), 0.5f);
    const dfl vc2 = dfl_scale(dfl_add(A.v[2][kA], A.v[2][kB]), 0.5f);
    dfl hg;  // g_part(1) = g_part(2) = g/2 (pick_random_velocity_on_sphere :343-351)
    {
      const dfl t = dfl_from_double(gg);
      hg = dfl_scale(dfl_norm(t.hi, t.lo), 0.5f);
    }
    for (int r = 0; r < NR; ++r) {
      // the uniforms as 53-bit integers (Philox) or recorded doubles
      unsigned long long mphi = 0, mcos = 0;
      double rphi_rec = 0.0, rcos_rec = 0.0;
      if (rec) {
        rphi_rec = a.pairs.rphi[q][i * NR + r];
        rcos_rec = a.pairs.rcos[q][i * NR + r];
        mphi = u53_bits(rphi_rec);
      } else {
        sample_u53x2<kKeys, true>(a, static_cast<uint32_t>(i), cell, step, q, 1u + r, mphi, mcos);
      }
      // phi = 2 pi R (pick_random_velocity_on_sphere :284-352): R = k/kTrigN + t, cos and
      // sin of 2 pi k/kTrigN from the table, of th = 2 pi t (< 0.0062) by Taylor series
      // (the dropped terms are below 1e-17), then the angle-addition formulas
      dfl cphi, sphi;
      {
        int k;
        const dfl th = dfl_mul(two_pi, angle_fraction(mphi, k));
        const dfl t2 = dfl_mul(th, th);
        const float t2h = t2.hi;
        // sin th = th - th (t2/6 - t2^2/120), cos th = 1 - (t2/2 - t2^2/24 + t2^3/720)
        const dfl cs1 = dfl_sub(dfl_mul(t2, one_sixth), dfl_make(t2h * t2h * (1.f / 120.f), 0.f));
        const dfl sth = dfl_sub(th, dfl_mul(th, cs1));
        const dfl cc1 = dfl_sub(dfl_scale(t2, 0.5f),
                                dfl_make(t2h * t2h * (1.f / 24.f - t2h * (1.f / 720.f)), 0.f));
        const dfl cth = dfl_sub(dfl_make(1.f, 0.f), cc1);
        const float4 tb = strig[min(max(k, 0), kTrigN - 1)];
        const dfl C = dfl_make(tb.x, tb.y), S = dfl_make(tb.z, tb.w);
        cphi = dfl_sub(dfl_mul(C, cth), dfl_mul(S, sth));
        sphi = dfl_add(dfl_mul(S, cth), dfl_mul(C, sth));
      }
      dfl ux, uy, uz;  // r / 2: half the post-collision relative velocity
      if (vss) {
        // VSS branch (pick_random_velocity_on_sphere :314-328) in pairs: cos theta =
        // 2 R^(1/alpha) - 1 by dfl_pow; |x_A - v0| + |x_B - v0| = |x_A - x_B| for the midpoint
        // v0 of a like-species pair
        const dfl ur = dfl_abs(dfl_sub(A.v[0][iA], A.v[0][iB]));
        const dfl vr_ = dfl_abs(dfl_sub(A.v[1][jA], A.v[1][jB]));
        const dfl wr = dfl_abs(dfl_sub(A.v[2][kA], A.v[2][kB]));
        dfl ct = dfl_make(-1.f, 0.f);  // R = 0
        {
          const double rc = rec ? rcos_rec : u53m(mcos);
          if (rc > 0.0) {
            const dfl r = dfl_from_double(rc);
            const float2 qa = sexp2[kExp2TabN + 2], qb = sexp2[kExp2TabN + 3];
            flt3 q;
            q.hi = qa.x; q.mid = qa.y; q.lo = qb.x;
            ct = dfl_sub(dfl_scale(dfl_pow(dfl_norm(r.hi, r.lo), q, sexp2), 2.f),
                         dfl_make(1.f, 0.f));
          }
        }
        const dfl one = dfl_make(1.f, 0.f);
        const dfl stt = dfl_sqrt(dfl_sub(one, dfl_mul(ct, ct)));
        const dfl den = dfl_sqrt(dfl_add(dfl_mul(vr_, vr_), dfl_mul(wr, wr)));
        const dfl gp = dfl_scale(hg, 2.f);  // |g|
        dfl rx, ry, rz;
        if (den.hi > static_cast<float>(kDoubleTol) * gp.hi) {
          rx = dfl_add(dfl_mul(ct, ur), dfl_mul(dfl_mul(stt, sphi), den));
          const dfl ny = dfl_sub(dfl_mul(dfl_mul(gp, wr), cphi), dfl_mul(dfl_mul(ur, vr_), sphi));
          const dfl nz = dfl_add(dfl_mul(dfl_mul(gp, vr_), cphi), dfl_mul(dfl_mul(ur, wr), sphi));
          ry = dfl_add(dfl_mul(ct, vr_), dfl_div(dfl_mul(stt, ny), den));
          rz = dfl_sub(dfl_mul(ct, wr), dfl_div(dfl_mul(stt, nz), den));
        } else {
          rx = dfl_mul(ct, ur);
          ry = dfl_mul(dfl_mul(stt, cphi), ur);
          rz = dfl_mul(dfl_mul(stt, sphi), ur);
        }
        ux = dfl_scale(rx, 0.5f); uy = dfl_scale(ry, 0.5f); uz = dfl_scale(rz, 0.5f);
      } else {
        // cos theta = 2 R - 1 (exact in FP64), sin theta = sqrt(1 - cos^2)
        dfl ct;
        {
          // 2 R - 1, exact: from the recorded double, or as (2 m - 2^53) 2^-53
          const double x = rec ? fma(2.0, rcos_rec, -1.0)
                               : static_cast<double>(static_cast<long long>(2 * mcos) -
                                                     (1ll << 53)) * 0x1.0p-53;
          const dfl t = dfl_from_double(x);
          ct = dfl_norm(t.hi, t.lo);
        }
        const dfl stt = dfl_sqrt(dfl_sub(dfl_make(1.f, 0.f), dfl_mul(ct, ct)));
        const dfl hs = dfl_mul(hg, stt);
        ux = dfl_mul(hs, cphi);
        uy = dfl_mul(hs, sphi);
        uz = dfl_mul(hg, ct);
      }
      // both velocities are formed before the first scatter (the centre of mass and the
      // relative half-velocity are not live across it) and go through one copy of the
      // remap in a two-pass loop: two inlined copies made the kernel wait on instruction
      // fetch
      dfl q0 = dfl_add(vc0, ux), q1 = dfl_add(vc1, uy), q2 = dfl_add(vc2, uz);
      const dfl pB0 = dfl_sub(vc0, ux), pB1 = dfl_sub(vc1, uy), pB2 = dfl_sub(vc2, uz);
#pragma unroll 1
      for (int side = 0; side < 2; ++side) {
        const int rb = remap_scatter_dfl<kFast>(g, A, q0, q1, q2, a.vmin[0], a.vmin[1],
                                                a.vmin[2], a.vfac[0], a.vfac[1], a.vfac[2], f,
                                                kr, nat);
        if (rb & 2) bad |= DVM_EW_REMAP;
        if (rb & 1) bad |= DVM_EW_SEARCH;
        q0 = pB0; q1 = pB1; q2 = pB2;
      }
    }
    }  // the run's chunks
  }
  if (bad) atomicOr(a.err, bad);
  add_scatter_count(a.scatter_count, nat);
}

// Four CTAs per SM (64 registers): the kernel needs the warps more than the registers
// (three CTAs at 80 registers measured 5.55 against 5.47 ms for the general kernel, 4.34
// against 4.19 ms for the common configuration's copy on the benchmark shock; five at 48
// registers 5.22 against 5.05 ms).
template <bool kFast>
__global__ void __launch_bounds__(kCollideChunk, 4) k_collide(CollideArgs a) {
  collide_cta<kFast, true>(a, blockIdx.x, gridDim.x);
}

size_t collide_smem_bytes(const GridInfo& g, const CollTables& t) {
  return collide_smem_layout(g, t).total;
}

int collide_blocks_per_sm(size_t smem) {
  int n = 0;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_collide<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_collide<false>, kCollideChunk, smem) !=
      cudaSuccess)
    n = 1;
  cudaGetLastError();  // a refused query must not surface at the next launch
  return n > 0 ? n : 1;
}

// The FP32 grid constants of the collide kernels, formed on the host.
static CollideArgs with_collide_consts(const CollideArgs& a) {
  CollideArgs b = a;
  b.vmin[0] = static_cast<float>(a.g.xv_min);
  b.vmin[1] = static_cast<float>(a.g.yv_min);
  b.vmin[2] = static_cast<float>(a.g.zv_min);
  b.vfac[0] = static_cast<float>(a.g.xv_factor);
  b.vfac[1] = static_cast<float>(a.g.yv_factor);
  b.vfac[2] = static_cast<float>(a.g.zv_factor);
  b.rnx = 1.f / static_cast<float>(a.g.nx);
  b.rnxy = 1.f / static_cast<float>(a.g.nx * a.g.ny);
  philox_key_schedule(a.cp.seed, b.rk);
  return b;
}

CollideArgs collide_consts(const CollideArgs& a) { return with_collide_consts(a); }

cudaError_t launch_collide(const CollideArgs& a, int grid, cudaStream_t s) {
  const size_t smem = collide_smem_bytes(a.g, a.t);
  const bool fast = collide_fast(a);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(
        k_collide<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_collide<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  if (fast) k_collide<true><<<grid, kCollideChunk, smem, s>>>(with_collide_consts(a));
  else k_collide<false><<<grid, kCollideChunk, smem, s>>>(with_collide_consts(a));
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// Precision form: k_collide_f32 draws the same partners as k_collide (FP64 CDFs, integer
// compares, the same Philox words) but forms the post-collision velocities, remap weights
// and contributions in FP32 and scatters them into an FP32 increment df; k_project then
// adds df to f in FP64 after removing, per cell, the weighted least-norm correction that
// makes the increment conserve mass, momentum and energy exactly.
struct StencilF {
  int node[7];
  float mass[7];
};

__device__ __forceinline__ int okeyf(float d) {
  int b = __float_as_int(d);
  if (b == static_cast<int>(0x80000000u)) b = 0;
  return b >= 0 ? b : (b ^ 0x7FFFFFFF);
}

struct SmemAxesF {
  const float* v[3];
  const int* mid[3];
  const AxisEntryF* tab[3];
  int n[3];
};

__device__ __forceinline__ void find_boundary_stencil_f(int& sa, int& sb, int& sc, float abc,
                                                        int oi, int oj, int ok, const float* x,
                                                        const float* y, const float* z,
                                                        int i_max, int j_max, int k_max) {
  while (oi + sa > 0 && oi + sa < i_max) {
    if (fabsf(abc) > 0.5f * fabsf(x[oi + sa] - x[oi])) sa = sa + isign1(sa);
    else break;
  }
  while (oj + sb > 0 && oj + sb < j_max && oj - sb > 0 && oj - sb < j_max) {
    if (fabsf(abc) > 0.5f * fabsf(y[oj + sb] - y[oj])) sb = sb + isign1(sb);
    else break;
  }
  while (ok + sc > 0 && ok + sc < k_max && ok - sc > 0 && ok - sc < k_max) {
    if (fabsf(abc) > 0.5f * fabsf(z[ok + sc] - z[ok])) sc = sc + isign1(sc);
    else break;
  }
}

__device__ __forceinline__ int nearest_f(const SmemAxesF& A, int ax, float u, float vmin,
                                         float factor, int& corner, int& bad) {
  const int mx = A.n[ax] - 1;
  const int* mid = A.mid[ax];
  const int vk = okeyf(u);
  int o = round_small(factor * (u - vmin));
  o = o < 0 ? 0 : (o > mx ? mx : o);
  if (u != u) bad |= 1;
  int it = 0;
  while (o > 0 && vk <= mid[o - 1] && it++ < kMaxAxis) --o;
  while (o < mx && vk > mid[o] && it++ < kMaxAxis) ++o;
  if (o >= mx) { o = mx; corner++; }
  else if (o <= 0) { o = 0; corner++; }
  return o;
}

// compute_remapping_quantities (collisions/remapping.f90:92-394) in FP32.
__device__ __forceinline__ int remap_f32(const GridInfo& g, const float (&vmin)[3],
                                         const float (&vfac)[3], const SmemAxesF& A, float u,
                                         float v, float w, StencilF& s) {
  int corner = 0, bad = 0;
  int o_i = nearest_f(A, 0, u, vmin[0], vfac[0], corner, bad);
  int o_j = nearest_f(A, 1, v, vmin[1], vfac[1], corner, bad);
  int o_k = nearest_f(A, 2, w, vmin[2], vfac[2], corner, bad);
  const int i_max = g.nx - 1, j_max = g.ny - 1, k_max = g.nz - 1;
  if (corner == 3) {
    o_i -= isign1(o_i - 1);
    o_j -= isign1(o_j - 1);
    o_k -= isign1(o_k - 1);
  }
  const float* x = A.v[0];
  const float* y = A.v[1];
  const float* z = A.v[2];
  const float ox = x[o_i], oy = y[o_j], oz = z[o_k];
  const float a = u - ox, b = v - oy, c = w - oz;
  int sa = signbit(a) ? -1 : 1, sb = signbit(b) ? -1 : 1, sc = signbit(c) ? -1 : 1;
  if (o_i + sa > i_max || o_i + sa < 0) {
    sa = -sa;
    find_boundary_stencil_f(sa, sb, sc, a, o_i, o_j, o_k, x, y, z, i_max, j_max, k_max);
  }
  if (o_j + sb > j_max || o_j + sb < 0) {
    sb = -sb;
    find_boundary_stencil_f(sb, sa, sc, b, o_j, o_i, o_k, y, x, z, j_max, i_max, k_max);
  }
  if (o_k + sc > k_max || o_k + sc < 0) {
    sc = -sc;
    find_boundary_stencil_f(sc, sb, sa, c, o_k, o_j, o_i, z, y, x, k_max, j_max, i_max);
  }
  const int fx = (o_i - sa <= i_max && o_i - sa >= 0);
  const int fy = (o_j - sb <= j_max && o_j - sb >= 0);
  const int fz = (o_k - sc <= k_max && o_k - sc >= 0);
  float int_x, inv_x, ext_x = 0.f, t_x = 0.f;
  if (sa >= -kTabS && sa <= kTabS) {
    const AxisEntryF& e = A.tab[0][o_i];
    int_x = e.D[kTabS + sa]; inv_x = e.invD[kTabS + sa];
    if (fx) { ext_x = e.D[kTabS - sa]; t_x = e.T[kTabS + sa]; }
  } else {
    int_x = x[o_i + sa] - ox; inv_x = 1.f / int_x;
    if (fx) { ext_x = x[o_i - sa] - ox; t_x = ext_x * (ext_x - int_x); }
  }
  float int_y, inv_y, ext_y = 0.f, t_y = 0.f;
  if (sb >= -kTabS && sb <= kTabS) {
    const AxisEntryF& e = A.tab[1][o_j];
    int_y = e.D[kTabS + sb]; inv_y = e.invD[kTabS + sb];
    if (fy) { ext_y = e.D[kTabS - sb]; t_y = e.T[kTabS + sb]; }
  } else {
    int_y = y[o_j + sb] - oy; inv_y = 1.f / int_y;
    if (fy) { ext_y = y[o_j - sb] - oy; t_y = ext_y * (ext_y - int_y); }
  }
  float int_z, inv_z, ext_z = 0.f, t_z = 0.f;
  if (sc >= -kTabS && sc <= kTabS) {
    const AxisEntryF& e = A.tab[2][o_k];
    int_z = e.D[kTabS + sc]; inv_z = e.invD[kTabS + sc];
    if (fz) { ext_z = e.D[kTabS - sc]; t_z = e.T[kTabS + sc]; }
  } else {
    int_z = z[o_k + sc] - oz; inv_z = 1.f / int_z;
    if (fz) { ext_z = z[o_k - sc] - oz; t_z = ext_z * (ext_z - int_z); }
  }
  const float den = (fx ? t_x : 0.f) + (fy ? t_y : 0.f) + (fz ? t_z : 0.f);
  float f_e = 0.f;
  if (!(fx | fy | fz)) bad |= 2;
  else f_e = __fdividef(a * a + b * b + c * c - a * int_x - b * int_y - c * int_z, den);
  const float f_ex = fx ? f_e : 0.f, f_ey = fy ? f_e : 0.f, f_ez = fz ? f_e : 0.f;
  const float f_ix = (a - f_ex * ext_x) * inv_x;
  const float f_iy = (b - f_ey * ext_y) * inv_y;
  const float f_iz = (c - f_ez * ext_z) * inv_z;
  const float f_o = 1.f - f_ix - f_iy - f_iz - f_ex - f_ey - f_ez;
  const int NX = g.nx, NXY = g.nx * g.ny;
  const int base = o_i + NX * o_j + NXY * o_k;
  s.node[0] = base;
  s.node[1] = base + sa;
  s.node[2] = base + NX * sb;
  s.node[3] = base + NXY * sc;
  s.node[4] = fx ? base - sa : -1;
  s.node[5] = fy ? base - NX * sb : -1;
  s.node[6] = fz ? base - NXY * sc : -1;
  s.mass[0] = f_o; s.mass[1] = f_ix; s.mass[2] = f_iy; s.mass[3] = f_iz;
  s.mass[4] = f_ex; s.mass[5] = f_ey; s.mass[6] = f_ez;
  return bad;
}

// FP32 reductions of 2 or 4 adjacent floats in one L2 transaction (the address aligned to
// 8 or 16 bytes).
__device__ __forceinline__ void red_add_v2(float* p, float a, float b) {
  asm volatile("red.global.add.v2.f32 [%0], {%1, %2};" ::"l"(__cvta_generic_to_global(p)),
               "f"(a), "f"(b) : "memory");
}
__device__ __forceinline__ void red_add_v4(float* p, float a, float b, float c, float d) {
  asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(__cvta_generic_to_global(p)),
               "f"(a), "f"(b), "f"(c), "f"(d) : "memory");
}

// Adds w * mass at a stencil's nodes into the FP32 increment df of one cell. The adds run at
// the L2 transaction rate whatever their type, so the three x-neighbours (base - 1, base,
// base + 1, adjacent in memory) go out as one 16-byte or one 8-byte plus one 4-byte
// reduction when the slab is 16-byte aligned (vec) and the x-stencil is the adjacent one;
// absent nodes inside an aligned group receive 0. Returns the nodes written.
__device__ __forceinline__ int scatter_stencil_f32(float* df, const StencilF& s, float w,
                                                   bool vec) {
  int n = 0;
  const int b = s.node[0];
  const int sa = s.node[1] - b;  // +-1, or wider next to a grid edge (find_boundary_stencil)
  if (vec && (sa == 1 || sa == -1)) {
    const bool ex = s.node[4] >= 0;
    const float v0 = w * s.mass[0], vi = w * s.mass[1], ve = ex ? w * s.mass[4] : 0.f;
    const float vm = sa > 0 ? ve : vi, vp = sa > 0 ? vi : ve;  // at b - 1 and b + 1
    float* q = df + (b & ~3);
    switch (b & 3) {
      case 1: red_add_v4(q, vm, v0, vp, 0.f); break;
      case 2: red_add_v4(q, 0.f, vm, v0, vp); break;
      case 0:
        red_add_v2(df + b, v0, vp);
        if (sa < 0 || ex) atomicAdd(df + b - 1, vm);
        break;
      default:
        red_add_v2(df + b - 1, vm, v0);
        if (sa > 0 || ex) atomicAdd(df + b + 1, vp);
        break;
    }
    n = ex ? 3 : 2;
  } else {
#pragma unroll
    for (int m = 0; m < 2; ++m) { atomicAdd(df + s.node[m], w * s.mass[m]); ++n; }
    if (s.node[4] >= 0) { atomicAdd(df + s.node[4], w * s.mass[4]); ++n; }
  }
  atomicAdd(df + s.node[2], w * s.mass[2]);
  atomicAdd(df + s.node[3], w * s.mass[3]);
  n += 2;
  if (s.node[5] >= 0) { atomicAdd(df + s.node[5], w * s.mass[5]); ++n; }
  if (s.node[6] >= 0) { atomicAdd(df + s.node[6], w * s.mass[6]); ++n; }
  return n;
}

struct CollideSmemF {
  size_t axes, keys, tabs, gtab, trig, total;
};

__host__ __device__ inline CollideSmemF collide_f32_smem_layout(const GridInfo& g,
                                                                const CollTables& t,
                                                                int gtab_smem) {
  CollideSmemF L;
  const size_t nsum = static_cast<size_t>(g.nx + g.ny + g.nz);
  L.axes = 0;
  L.keys = L.axes + nsum * sizeof(float);
  L.tabs = (L.keys + nsum * sizeof(int) + 15) & ~static_cast<size_t>(15);
  L.gtab = (L.tabs + 3 * static_cast<size_t>(t.nmax) * sizeof(AxisEntryF) + 15) &
           ~static_cast<size_t>(15);
  L.trig = L.gtab + (gtab_smem ? static_cast<size_t>(t.gtab_n) * sizeof(float2) : 0);
  L.total = L.trig + static_cast<size_t>(kTrigN) * sizeof(float2);
  return L;
}

// Shared-memory tables of the FP32 collide kernels.
struct F32Ctx {
  SmemAxesF A;
  const float2* gtab;
  const float2* strig;
  float vhs, ralpha;
  bool vss, vr;
  int NR;
  uint32_t step;
};

__device__ __forceinline__ F32Ctx load_f32_tables(const CollideArgs& a, const CollTablesF& tf,
                                                  unsigned char* s_raw) {
  const GridInfo& g = a.g;
  const CollideSmemF L = collide_f32_smem_layout(g, a.t, tf.gtab_smem);
  float* sv = reinterpret_cast<float*>(s_raw + L.axes);
  int* sk = reinterpret_cast<int*>(s_raw + L.keys);
  AxisEntryF* st = reinterpret_cast<AxisEntryF*>(s_raw + L.tabs);
  float2* sg = reinterpret_cast<float2*>(s_raw + L.gtab);
  float2* strig = reinterpret_cast<float2*>(s_raw + L.trig);
  const int nsum = g.nx + g.ny + g.nz;
  for (int t = threadIdx.x; t < nsum; t += blockDim.x) {
    const double* ax = t < g.nx ? g.x : (t < g.nx + g.ny ? g.y : g.z);
    const int n = t < g.nx ? g.nx : (t < g.nx + g.ny ? g.ny : g.nz);
    const int i = t < g.nx ? t : (t < g.nx + g.ny ? t - g.nx : t - g.nx - g.ny);
    sv[t] = static_cast<float>(ax[i]);
    sk[t] = (i + 1 < n) ? okeyf(static_cast<float>(0.5 * (ax[i] + ax[i + 1]))) : 0x7FFFFFFF;
  }
  {
    const float* src = reinterpret_cast<const float*>(tf.axis);
    float* dst = reinterpret_cast<float*>(st);
    const int n = 3 * a.t.nmax * static_cast<int>(sizeof(AxisEntryF) / sizeof(float));
    for (int t = threadIdx.x; t < n; t += blockDim.x) dst[t] = src[t];
  }
  if (tf.gtab_smem)
    for (int t = threadIdx.x; t < a.t.gtab_n; t += blockDim.x) sg[t] = tf.gtab[t];
  for (int t = threadIdx.x; t < kTrigN; t += blockDim.x) strig[t] = tf.trig[t];
  F32Ctx c;
  c.A.v[0] = sv; c.A.v[1] = sv + g.nx; c.A.v[2] = sv + g.nx + g.ny;
  c.A.mid[0] = sk; c.A.mid[1] = sk + g.nx; c.A.mid[2] = sk + g.nx + g.ny;
  c.A.tab[0] = st; c.A.tab[1] = st + a.t.nmax; c.A.tab[2] = st + 2 * a.t.nmax;
  c.A.n[0] = g.nx; c.A.n[1] = g.ny; c.A.n[2] = g.nz;
  c.gtab = a.t.gtab ? (tf.gtab_smem ? sg : tf.gtab) : nullptr;
  c.strig = strig;
  c.vhs = static_cast<float>(2.0 - 2.0 * (0.5 * (a.cp.omega + a.cp.omega)));
  c.ralpha = 1.f / static_cast<float>(0.5 * (a.cp.alpha + a.cp.alpha));
  c.vss = fabs(1.0 / (0.5 * (a.cp.alpha + a.cp.alpha)) - 1.0) > kDoubleTol;
  c.vr = (a.cp.method == DVM_COLL_VR);
  c.NR = a.cp.num_repl;
  c.step = a.step_dev ? *a.step_dev : a.step;
  return c;
}

// One sample of sub-integral q of a cell in FP32, scattered into df (global or shared).
template <bool kFast, bool kKeys>
__device__ __forceinline__ void collide_sample_f32(const CollideArgs& a, const CollTablesF& tf,
                                                   const F32Ctx& c, int cell, int q, long long i,
                                                   float factor, float* df, uint32_t& bad,
                                                   uint32_t& nat) {
  const GridInfo& g = a.g;
  const SmemAxesF& A = c.A;
  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const size_t cs = static_cast<size_t>(cell) * (nv + 1);
  const bool vr = c.vr;
  unsigned long long mA = 0, mB = 0;
  const bool rec = kFast ? false : a.pairs.active;
  if (!rec) sample_u53x2<kKeys>(a, static_cast<uint32_t>(i), cell, c.step, q, 0u, mA, mB);
  int lA, lB;
  if (rec && a.pairs.glA[q]) {
    lA = a.pairs.glA[q][i];
    lB = a.pairs.glB[q][i];
  } else {
    bool tA = mA < kTolU53, tB = mB < kTolU53;
    if (rec) {
      const double rA = a.pairs.rA[q][i], rB = a.pairs.rB[q][i];
      mA = u53_bits(rA); mB = u53_bits(rB);
      tA = __double_as_longlong(rA) < __double_as_longlong(kDoubleTol);
      tB = __double_as_longlong(rB) < __double_as_longlong(kDoubleTol);
    }
    const bool aeq = vr && q == 0, beq = vr && q == 1;
    lA = referenced_search_fixed((aeq ? a.cum_eq : a.cum_dev) + cs,
                                 (aeq ? a.ref_eq : a.ref_dev) + static_cast<size_t>(cell) * kNRef,
                                 nv, mA, tA, bad);
    lB = referenced_search_fixed((beq ? a.cum_eq : a.cum_dev) + cs,
                                 (beq ? a.ref_eq : a.ref_dev) + static_cast<size_t>(cell) * kNRef,
                                 nv, mB, tB, bad);
  }
  int iA, jA, kA, iB, jB, kB;
  node_ijk(lA, NX, NXY, a.rnx, a.rnxy, iA, jA, kA);
  node_ijk(lB, NX, NXY, a.rnx, a.rnxy, iB, jB, kB);
  const float xA = A.v[0][iA], yA = A.v[1][jA], zA = A.v[2][kA];
  const float xB = A.v[0][iB], yB = A.v[1][jB], zB = A.v[2][kB];
  float gg, g_sigma;
  if (kFast || c.gtab) {
    const int di = iB - iA, dj = jB - jA, dk = kB - kA;
    const int s2 = di * di + dj * dj + dk * dk;
    if (s2 == 0) return;
    const float2 e = c.gtab[s2];
    gg = e.x;
    g_sigma = e.y;
  } else {
    const float gx = xB - xA, gy = yB - yA, gz = zB - zA;
    gg = sqrtf(gx * gx + gy * gy + gz * gz);
    if (gg < 1e-13f) return;
    g_sigma = (c.vhs == 1.f) ? gg : powf(gg, c.vhs);
  }
  const float sA = (vr && q == 0) ? 1.f : ((__ldg(a.cum_dev + cs + lA + 1) & 1) ? -1.f : 1.f);
  const float sB = (vr && q == 1) ? 1.f : ((__ldg(a.cum_dev + cs + lB + 1) & 1) ? -1.f : 1.f);
  const float kin = sA * sB * factor * g_sigma;
  atomicAdd(df + lA, -kin);
  atomicAdd(df + lB, -kin);
  nat += 2u;
  const int NR = kFast ? 1 : c.NR;
  const float kr = kFast ? kin : kin / static_cast<float>(NR);
  const float vc0 = 0.5f * (xA + xB), vc1 = 0.5f * (yA + yB), vc2 = 0.5f * (zA + zB);
  const float hg = 0.5f * gg;
  for (int r = 0; r < NR; ++r) {
    float rphi, rcos;
    if (rec) {
      rphi = static_cast<float>(a.pairs.rphi[q][i * NR + r]);
      rcos = static_cast<float>(a.pairs.rcos[q][i * NR + r]);
    } else {
      // the top 24 bits of the two uniforms the FP64 form draws from this counter
      uint32_t o[4];
      if (kKeys)
        philox4x32_10_rk(static_cast<uint32_t>(i), cell, c.step, (q & 3u) | ((1u + r) << 2),
                         a.rk, o);
      else
        philox4x32_10(static_cast<uint32_t>(i), cell, c.step, (q & 3u) | ((1u + r) << 2),
                      static_cast<uint32_t>(a.cp.seed), static_cast<uint32_t>(a.cp.seed >> 32),
                      o);
      rphi = static_cast<float>(o[1] >> 8) * 0x1.0p-24f;
      rcos = static_cast<float>(o[3] >> 8) * 0x1.0p-24f;
    }
    float sphi, cphi;
    {
      const float rk = floorf(rphi * static_cast<float>(kTrigN));
      const int k = min(max(static_cast<int>(rk), 0), kTrigN - 1);
      const float th = tf.two_pi * (rphi - rk * (1.f / kTrigN));
      const float t2 = th * th;
      const float st = th * (1.f - t2 * (1.f / 6.f));
      const float ct = 1.f - 0.5f * t2;
      const float2 cs2 = c.strig[k];
      cphi = cs2.x * ct - cs2.y * st;
      sphi = cs2.y * ct + cs2.x * st;
    }
    float ux, uy, uz;
    if (!kFast && c.vss) {
      const float ur = fabsf(xA - vc0) + fabsf(xB - vc0);
      const float vr_ = fabsf(yA - vc1) + fabsf(yB - vc1);
      const float wr = fabsf(zA - vc2) + fabsf(zB - vc2);
      const float ct = 2.f * powf(rcos, c.ralpha) - 1.f;
      const float stt = sqrtf(fmaxf(1.f - ct * ct, 0.f));
      const float den = sqrtf(vr_ * vr_ + wr * wr);
      float rx, ry, rz;
      if (den > 1e-13f * gg) {
        rx = ct * ur + stt * sphi * den;
        ry = ct * vr_ + stt * (gg * wr * cphi - ur * vr_ * sphi) / den;
        rz = ct * wr - stt * (gg * vr_ * cphi + ur * wr * sphi) / den;
      } else {
        rx = ct * ur; ry = stt * cphi * ur; rz = stt * sphi * ur;
      }
      ux = 0.5f * rx; uy = 0.5f * ry; uz = 0.5f * rz;
    } else {
      const float ct = 2.f * rcos - 1.f;
      const float stt = sqrtf(fmaxf(1.f - ct * ct, 0.f));
      ux = hg * stt * cphi;
      uy = hg * stt * sphi;
      uz = hg * ct;
    }
    // the cell's slab of df is 16-byte aligned when the node count is a multiple of 4
    const bool vec = (g.nv & 3) == 0;
    StencilF sA_, sB_;
    int rb = remap_f32(g, a.vmin, a.vfac, A, vc0 + ux, vc1 + uy, vc2 + uz, sA_);
    if (rb & 2) bad |= DVM_EW_REMAP;
    else nat += scatter_stencil_f32(df, sA_, kr, vec);
    rb = remap_f32(g, a.vmin, a.vfac, A, vc0 - ux, vc1 - uy, vc2 - uz, sB_);
    if (rb & 2) bad |= DVM_EW_REMAP;
    else nat += scatter_stencil_f32(df, sB_, kr, vec);
  }
}

// One CTA of the persistent FP32 collide launch (as collide_cta).
template <bool kFast, bool kKeys>
__device__ __forceinline__ void collide_f32_cta(const CollideArgs& a, const CollTablesF& tf,
                                                float* __restrict__ dfs, int bid, int nblk) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  const F32Ctx c = load_f32_tables(a, tf, s_raw);
  __syncthreads();
  const int nv = a.g.nv;
  const int nent = 3 * a.ncells;
  const long long total = a.chunk_off[nent] & kRunMask;
  const int runlen = static_cast<int>(a.chunk_off[nent] >> kRunShift);
  uint32_t bad = 0;
  uint32_t nat = 0;  // FP32 adds into df by this thread
  const int wpb = blockDim.x >> 5;
  const long long pos0 = static_cast<long long>(bid) * wpb + (threadIdx.x >> 5);
  const long long stride = static_cast<long long>(nblk) * wpb;
  ChunkWalk walk(pos0, stride, total);
  for (long long pos = pos0; pos < total; pos += stride) {
    const long long chunk = walk.next(total);
    int lo = 0, hi = nent;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (a.chunk_off[mid] <= chunk) lo = mid; else hi = mid;
    }
    const int cell = lo / 3, q = lo - 3 * (lo / 3);
    const CellPlan& pl = a.plan[cell];
    const long long i0 =
        (chunk - a.chunk_off[lo]) * (kChunkSamples * runlen) + (threadIdx.x & 31);
    for (int rr = 0; rr < runlen; ++rr) {
      const long long i = i0 + rr * kChunkSamples;
      if (i >= pl.num[q]) break;
      collide_sample_f32<kFast, kKeys>(a, tf, c, cell, q, i, static_cast<float>(pl.factor[q]),
                         dfs + static_cast<size_t>(cell) * nv, bad, nat);
    }
  }
  if (bad) atomicOr(a.err, bad);
  add_scatter_count(a.scatter_count, nat);
}

// The general kernel at three CTAs per SM: 80 registers hold the FP32 sample without
// spilling (3.25 against 3.32 ms at four CTAs and 64 registers on the benchmark shock).
// The common configuration's copy at four: 3.09 ms on the shock either way, 0.231 against
// 0.252 ms on the cavity, whose collide waits on DRAM and needs the warps.
template <bool kFast>
__global__ void __launch_bounds__(kCollideChunk, kFast ? 4 : 3) k_collide_f32(CollideArgs a, CollTablesF tf,
                                                                float* __restrict__ dfs) {
  collide_f32_cta<kFast, true>(a, tf, dfs, blockIdx.x, gridDim.x);
}

int collide_f32_blocks_per_sm(const GridInfo& g, const CollTables& t, bool fast) {
  const int gtab_smem = (t.gtab && static_cast<size_t>(t.gtab_n) * sizeof(float2) <= 48 * 1024) ? 1 : 0;
  const size_t smem = collide_f32_smem_layout(g, t, gtab_smem).total;
  const void* fn = fast ? reinterpret_cast<const void*>(k_collide_f32<true>)
                        : reinterpret_cast<const void*>(k_collide_f32<false>);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kCollideChunk, smem) != cudaSuccess)
    n = 1;
  cudaGetLastError();
  return n > 0 ? n : 1;
}

cudaError_t launch_collide_f32(const CollideArgs& a, const CollTablesF& tf, float* df, int grid,
                               cudaStream_t s) {
  const size_t smem = collide_f32_smem_layout(a.g, a.t, tf.gtab_smem).total;
  const bool fast = collide_fast(a);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k_collide_f32<false>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         static_cast<int>(smem));
    if (e == cudaSuccess)
      e = cudaFuncSetAttribute(k_collide_f32<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                               static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  if (fast) k_collide_f32<true><<<grid, kCollideChunk, smem, s>>>(with_collide_consts(a), tf, df);
  else k_collide_f32<false><<<grid, kCollideChunk, smem, s>>>(with_collide_consts(a), tf, df);
  return cudaGetLastError();
}

// k_project: one CTA per cell. With phi = (1, c_x, c_y, c_z, |c|^2), c = xi - u_cell, and
// weights w = |df|, the increment df - w * sum_k lambda_k phi_k with M lambda = r,
// M_kl = sum w phi_k phi_l, r_k = sum df phi_k, has zero mass, momentum and energy; it is
// the smallest such change in the w-weighted norm and vanishes where df does. The sums
// are taken column by column: per (i, j), sum_k of df z^p (p < 3) and of w z^p (p < 5).
//
// r must be FP64-accurate (it is the non-conservation being removed) and is summed in
// hi + lo float pairs; M only sets the shape of the correction, whose size is that of r,
// so FP32 sums suffice for it (a relative error e in M leaves e |r| unconserved, some
// 1e-16 of the cell's moments). The correction w * poly is formed in FP32 for the same
// reason, and f + df - w * poly is formed in FP64 from the exact doubles of the two floats.
constexpr int kProjThreads = 256;

// Threads per CTA of a kernel whose threads walk the (i, j) columns of one cell: the
// columns split into the fewest rounds of at most max_threads, each round a whole number
// of warps (576 columns of a 24^3 grid: 3 rounds of 192, no idle tail round).
static int column_threads(const GridInfo& g, int max_threads) {
  const int cols = g.nx * g.ny;
  const int rounds = (cols + max_threads - 1) / max_threads;
  const int per = (cols + rounds - 1) / rounds;
  return ((per + 31) / 32) * 32;
}

constexpr int kProjAhead1 = 8;  // column increments read ahead of the sums
constexpr int kProjAhead2 = 4;  // column nodes read ahead of the update

// The projection of one cell, for the block: df (global or shared) is read, its projected
// value added to f, and df zeroed when it is the global increment buffer.
__device__ __forceinline__ void project_cell(const GridInfo& g, float* df, bool zero_df,
                                             double* f, const double* P) {
  __shared__ float2 s_red[20 * 32];
  __shared__ float s_lam[5];
  __shared__ dfl s_axd[2 * kMaxAxis];  // x', y' as pairs
  __shared__ dfl s_zd[2 * kMaxAxis];   // z', z'^2 as pairs
  __shared__ float s_axf[2 * kMaxAxis];
  __shared__ float s_zf[4 * kMaxAxis];  // z'^p, p = 1..4
  const int NX = g.nx, NXY = g.nx * g.ny, NZ = g.nz;
  const double u = P[DVM_P_U], v = P[DVM_P_V], w = P[DVM_P_W];
  for (int t = threadIdx.x; t < NX; t += blockDim.x) {
    const double x = g.x[t] - u;
    s_axd[t] = dfl_from_double(x);
    s_axf[t] = static_cast<float>(x);
  }
  for (int t = threadIdx.x; t < g.ny; t += blockDim.x) {
    const double y = g.y[t] - v;
    s_axd[kMaxAxis + t] = dfl_from_double(y);
    s_axf[kMaxAxis + t] = static_cast<float>(y);
  }
  for (int t = threadIdx.x; t < NZ; t += blockDim.x) {
    const double z = g.z[t] - w;
    s_zd[t] = dfl_from_double(z);
    s_zd[kMaxAxis + t] = dfl_from_double(z * z);
    const float zf = static_cast<float>(z);
    s_zf[t] = zf;
    s_zf[kMaxAxis + t] = zf * zf;
    s_zf[2 * kMaxAxis + t] = zf * zf * zf;
    s_zf[3 * kMaxAxis + t] = (zf * zf) * (zf * zf);
  }
  __syncthreads();
  // 0-4: r (pairs); 5-19: M (row-major upper triangle, FP32 per thread)
  dacc acc[20];
#pragma unroll
  for (int q = 0; q < 20; ++q) dacc_zero(acc[q]);
  for (int col = threadIdx.x; col < NXY; col += blockDim.x) {
    dacc D0, D1, D2;
    dacc_zero(D0); dacc_zero(D1); dacc_zero(D2);
    float W0 = 0.f, W1 = 0.f, W2 = 0.f, W3 = 0.f, W4 = 0.f;
    // the column's increments are read kProjAhead1 nodes ahead of the sums
    float fb[kProjAhead1];
#pragma unroll
    for (int u = 0; u < kProjAhead1; ++u) fb[u] = (u < NZ) ? df[col + NXY * u] : 0.f;
    for (int k0 = 0; k0 < NZ; k0 += kProjAhead1) {
      float fn[kProjAhead1];
#pragma unroll
      for (int u = 0; u < kProjAhead1; ++u)
        fn[u] = (k0 + kProjAhead1 + u < NZ) ? df[col + NXY * (k0 + kProjAhead1 + u)] : 0.f;
#pragma unroll
      for (int u = 0; u < kProjAhead1; ++u) {
      const int k = k0 + u;
      if (k >= NZ) break;
      const float d = fb[u];
      if (d == 0.f) continue;
      const dfl dd = dfl_make(d, 0.f);
      dacc_add(D0, dd);
      dacc_fma(D1, dd, s_zd[k]);
      dacc_fma(D2, dd, s_zd[kMaxAxis + k]);
      const float wt = fabsf(d);
      W0 += wt;
      W1 = fmaf(wt, s_zf[k], W1);
      W2 = fmaf(wt, s_zf[kMaxAxis + k], W2);
      W3 = fmaf(wt, s_zf[2 * kMaxAxis + k], W3);
      W4 = fmaf(wt, s_zf[3 * kMaxAxis + k], W4);
      }
#pragma unroll
      for (int u = 0; u < kProjAhead1; ++u) fb[u] = fn[u];
    }
    const int j = col / NX, i = col - j * NX;
    const dfl X = s_axd[i], Y = s_axd[kMaxAxis + j];
    const dfl R = dfl_add(dfl_mul(X, X), dfl_mul(Y, Y));
    const dfl d0 = dfl_norm(D0.hi, D0.lo), d1 = dfl_norm(D1.hi, D1.lo);
    const dfl d2 = dfl_norm(D2.hi, D2.lo);
    dacc_add(acc[0], d0);
    dacc_fma(acc[1], d0, X);
    dacc_fma(acc[2], d0, Y);
    dacc_add(acc[3], d1);
    dacc_add(acc[4], dfl_add(dfl_mul(R, d0), d2));
    const float Xf = s_axf[i], Yf = s_axf[kMaxAxis + j];
    const float Rf = Xf * Xf + Yf * Yf;
    const float E0 = fmaf(Rf, W0, W2);  // sum w |c|^2
    const float m[15] = {W0, Xf * W0, Yf * W0, W1, E0,                     // M00..M04
                         Xf * Xf * W0, Xf * Yf * W0, Xf * W1, Xf * E0,     // M11..M14
                         Yf * Yf * W0, Yf * W1, Yf * E0,                   // M22..M24
                         W2, fmaf(Rf, W1, W3),                             // M33, M34
                         fmaf(Rf * Rf, W0, fmaf(2.f * Rf, W2, W4))};       // M44
#pragma unroll
    for (int q = 0; q < 15; ++q) acc[5 + q].hi += m[q];
  }
  double tot[20];
  {
    __shared__ float2 s_sum[20 * kProjThreads];
    block_sum_dfl_t<20>(acc, s_sum, s_red, tot);
  }
  if (threadIdx.x == 0) {
    // Cholesky of M in FP32; no correction if M is not positive definite (e.g. no
    // collisions landed in this cell). FP32 suffices: M only shapes the correction, whose
    // values are formed in FP32 anyway, and M lambda = r to FP32 rounding leaves some 1e-7
    // of a non-conservation that is itself some 1e-7 of the increment.
    float M[5][5], L[5][5] = {{0.f}}, y[5], lam[5];
    int m = 5;
    for (int r = 0; r < 5; ++r)
      for (int c = r; c < 5; ++c) {
        M[r][c] = static_cast<float>(tot[m]);
        M[c][r] = M[r][c];
        ++m;
      }
    bool ok = true;
    for (int r = 0; r < 5 && ok; ++r) {
      for (int c = 0; c <= r; ++c) {
        float sum = M[r][c];
        for (int k = 0; k < c; ++k) sum -= L[r][k] * L[c][k];
        if (r == c) {
          if (!(sum > 1e-30f)) { ok = false; break; }
          L[r][r] = sqrtf(sum);
        } else {
          L[r][c] = sum / L[c][c];
        }
      }
    }
    if (ok) {
      for (int r = 0; r < 5; ++r) {
        float sum = static_cast<float>(tot[r]);
        for (int k = 0; k < r; ++k) sum -= L[r][k] * y[k];
        y[r] = sum / L[r][r];
      }
      for (int r = 4; r >= 0; --r) {
        float sum = y[r];
        for (int k = r + 1; k < 5; ++k) sum -= L[k][r] * lam[k];
        lam[r] = sum / L[r][r];
      }
    } else {
      for (int r = 0; r < 5; ++r) lam[r] = 0.f;
    }
    for (int r = 0; r < 5; ++r) s_lam[r] = isfinite(lam[r]) ? lam[r] : 0.f;
  }
  __syncthreads();
  const float l0 = s_lam[0], l1 = s_lam[1], l2 = s_lam[2], l3 = s_lam[3], l4 = s_lam[4];
  for (int col = threadIdx.x; col < NXY; col += blockDim.x) {
    const int j = col / NX, i = col - j * NX;
    const float X = s_axf[i], Y = s_axf[kMaxAxis + j];
    const float base = fmaf(l4, X * X + Y * Y, fmaf(l2, Y, fmaf(l1, X, l0)));
    // increments and f read kProjAhead2 nodes ahead of the update
    float db[kProjAhead2];
    double fbb[kProjAhead2];
#pragma unroll
    for (int u = 0; u < kProjAhead2; ++u) {
      db[u] = (u < NZ) ? df[col + NXY * u] : 0.f;
      fbb[u] = (u < NZ) ? f[col + NXY * u] : 0.0;
    }
    for (int k0 = 0; k0 < NZ; k0 += kProjAhead2) {
      float dn[kProjAhead2];
      double fnn[kProjAhead2];
#pragma unroll
      for (int u = 0; u < kProjAhead2; ++u) {
        const int k = k0 + kProjAhead2 + u;
        dn[u] = (k < NZ) ? df[col + NXY * k] : 0.f;
        fnn[u] = (k < NZ) ? f[col + NXY * k] : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kProjAhead2; ++u) {
        const int k = k0 + u;
        if (k >= NZ) break;
        const int l = col + NXY * k;
        const float d = db[u];
        if (d == 0.f) continue;
        const float poly = fmaf(l4, s_zf[kMaxAxis + k], fmaf(l3, s_zf[k], base));
        const float corr = fabsf(d) * poly;
        f[l] = (fbb[u] + dbl_from_float_fast(d)) - dbl_from_float_fast(corr);
        if (zero_df) df[l] = 0.f;
      }
#pragma unroll
      for (int u = 0; u < kProjAhead2; ++u) { db[u] = dn[u]; fbb[u] = fnn[u]; }
    }
  }
}

__global__ void __launch_bounds__(kProjThreads, 3) k_project(ProjectArgs a) {
  const int cell = blockIdx.x;
  const size_t off = static_cast<size_t>(cell) * a.g.nv;
  project_cell(a.g, a.df + off, true, a.f + off, a.props + static_cast<size_t>(cell) * DVM_NPROP);
}

cudaError_t launch_project(const ProjectArgs& a, cudaStream_t s) {
  k_project<<<a.ncells, column_threads(a.g, kProjThreads), 0, s>>>(a);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// 2-D wall ghosts, conditions/boundary_conditions.f90:630-1527. Entry e is one wall side of
// one perimeter cell: sides in the order left, right, bottom, top.
struct WallEntry {
  int side, cx, cy;
};

__device__ __forceinline__ WallEntry wall_entry(const WallArgs& a, int e) {
  WallEntry w{-1, 0, 0};
  for (int s = 3; s >= 0; --s) {
    if (a.base[s] >= 0 && e >= a.base[s]) {
      w.side = s;
      const int pos = e - a.base[s];
      if (s == DVM_WALL_LEFT) { w.cx = 0; w.cy = pos; }
      else if (s == DVM_WALL_RIGHT) { w.cx = a.nxs - 1; w.cy = pos; }
      else if (s == DVM_WALL_BOTTOM) { w.cx = pos; w.cy = 0; }
      else { w.cx = pos; w.cy = a.nys - 1; }
      return w;
    }
  }
  return w;
}

// Incoming half of a wall (molecules moving into it) and its outgoing half.
__device__ __forceinline__ bool wall_incoming(const GridInfo& g, int side, int i, int j) {
  switch (side) {
    case DVM_WALL_LEFT: return i <= g.i_neg;
    case DVM_WALL_RIGHT: return i >= g.i_pos;
    case DVM_WALL_BOTTOM: return j <= g.j_neg;
    default: return j >= g.j_pos;
  }
}
__device__ __forceinline__ bool wall_outgoing(const GridInfo& g, int side, int i, int j) {
  switch (side) {
    case DVM_WALL_LEFT: return i >= g.i_pos;
    case DVM_WALL_RIGHT: return i <= g.i_neg;
    case DVM_WALL_BOTTOM: return j >= g.j_pos;
    default: return j <= g.j_neg;
  }
}

constexpr int kWallThreads = 512;

// Diffuse part: ghost = (flux_in/flux_out) * M(T_w, u_w) beta3 on the outgoing half
// (:763-828); zero elsewhere.
__global__ void __launch_bounds__(kWallThreads) k_wall_flux(WallArgs a) {
  __shared__ double s_red[2 * 32];
  __shared__ double s_fac[3 * kMaxAxis];
  const GridInfo& g = a.g;
  const WallEntry we = wall_entry(a, blockIdx.x);
  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const double* f = a.f + (static_cast<size_t>(we.cx) + static_cast<size_t>(a.nxs) * we.cy) * nv;
  double* gh = a.ghost + static_cast<size_t>(blockIdx.x) * nv;
  const bool xwall = (we.side == DVM_WALL_LEFT || we.side == DVM_WALL_RIGHT);
  const double* W = a.wall[we.side];
  const double T = W[DVM_WP_TEMP], u = W[DVM_WP_U], v = W[DVM_WP_V], w = W[DVM_WP_W];
  const double mc = maxwell_coeff(a.mass, T, a.pi);
  // the half-Maxwellian times the node volume factorises over the axes (:793-813)
  const int nsum = g.nx + g.ny + g.nz;
  for (int t = threadIdx.x; t < nsum; t += blockDim.x) {
    double c, b, sc = 1.0;
    int o;
    if (t < g.nx) { c = g.x[t] - u; b = g.bx[t]; sc = mc; o = t; }
    else if (t < g.nx + g.ny) { c = g.y[t - g.nx] - v; b = g.by[t - g.nx]; o = kMaxAxis + t - g.nx; }
    else { c = g.z[t - g.nx - g.ny] - w; b = g.bz[t - g.nx - g.ny]; o = 2 * kMaxAxis + t - g.nx - g.ny; }
    s_fac[o] = sc * exp(-(c * c) * a.mass / T) * b;
  }
  __syncthreads();
  double acc2[2] = {0.0, 0.0};  // flux_in, flux_out
  for (int l = threadIdx.x; l < nv; l += blockDim.x) {
    const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
    const double vn = xwall ? g.x[i] : g.y[j];
    if (wall_incoming(g, we.side, i, j)) acc2[0] += fabs(vn) * a.acc * f[l];
    double val = 0.0;
    if (a.acc > 0.0 && wall_outgoing(g, we.side, i, j)) {
      val = s_fac[i] * s_fac[kMaxAxis + j] * s_fac[2 * kMaxAxis + k];
      acc2[1] += fabs(vn) * val;
    }
    gh[l] = val;
  }
  block_sum<2>(acc2, s_red);
  if (a.acc > 0.0) {
    const double ratio = acc2[0] / acc2[1];
    for (int l = threadIdx.x; l < nv; l += blockDim.x) gh[l] = ratio * gh[l];
  }
}

// Specular part: each incoming node's (1-acc) f remapped at the mirrored velocity
// (:832-858, :1852-1929). Grid (entries, chunks of incoming nodes).
__global__ void __launch_bounds__(256) k_wall_spec(WallArgs a) {
  const GridInfo& g = a.g;
  const WallEntry we = wall_entry(a, blockIdx.x);
  const int nv = g.nv;
  const bool xwall = (we.side == DVM_WALL_LEFT || we.side == DVM_WALL_RIGHT);
  // incoming index range along the wall normal
  int lo, n_in;
  if (we.side == DVM_WALL_LEFT) { lo = 0; n_in = g.i_neg + 1; }
  else if (we.side == DVM_WALL_RIGHT) { lo = g.i_pos; n_in = g.nx - g.i_pos; }
  else if (we.side == DVM_WALL_BOTTOM) { lo = 0; n_in = g.j_neg + 1; }
  else { lo = g.j_pos; n_in = g.ny - g.j_pos; }
  if (n_in <= 0) return;
  const int t = blockIdx.y * blockDim.x + threadIdx.x;
  const int other = xwall ? g.ny : g.nx;
  if (t >= n_in * other * g.nz) return;
  int i, j, k;
  if (xwall) { i = lo + t % n_in; j = (t / n_in) % g.ny; k = t / (n_in * g.ny); }
  else { i = t % g.nx; j = lo + (t / g.nx) % n_in; k = t / (g.nx * n_in); }
  const int l = i + g.nx * j + g.nx * g.ny * k;
  const double* f = a.f + (static_cast<size_t>(we.cx) + static_cast<size_t>(a.nxs) * we.cy) * nv;
  double* gh = a.ghost + static_cast<size_t>(blockIdx.x) * nv;
  const double dens = (1.0 - a.acc) * f[l];
  Stencil s;
  const int rb = xwall ? remap(g, g.x, g.y, g.z, -g.x[i], g.y[j], g.z[k], 1.0, s)
                       : remap(g, g.x, g.y, g.z, g.x[i], -g.y[j], g.z[k], 1.0, s);
  if (rb & 2) { atomicOr(a.err, DVM_EW_REMAP); return; }
#pragma unroll
  for (int q = 0; q < 7; ++q)
    if (s.node[q] >= 0) atomicAdd(gh + s.node[q], dens * s.mass[q]);
}

cudaError_t launch_wall_flux(const WallArgs& a, cudaStream_t s) {
  if (a.nentries <= 0) return cudaSuccess;
  k_wall_flux<<<a.nentries, kWallThreads, 0, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_wall_specular(const WallArgs& a, cudaStream_t s) {
  if (a.nentries <= 0 || !(a.acc < 1.0)) return cudaSuccess;
  const GridInfo& g = a.g;
  const int nmax = g.nv;  // an upper bound of incoming nodes per entry
  dim3 grid(a.nentries, (nmax + 255) / 256);
  k_wall_spec<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// k_convect2d: every cell, every node. Interior cells: first_order_scheme
// (convection/convection.f90:119-276). Perimeter cells: the ghost update of
// set_boundary_nodes (:1552-1643), whose loops cover only the i/j ranges below; nodes they
// skip keep the zero that phi_conv was reset to (:694).
enum { kClsNone = 0, kClsNeg = 1, kClsPos = 2, kClsZero = 3 };

__device__ __forceinline__ int axis_class(int i, int neg, int pos, int zero, int zero_flag) {
  if (i <= neg) return kClsNeg;
  if (i >= pos) return kClsPos;
  if (zero_flag && i == zero) return kClsZero;
  return kClsNone;
}

// The update f0 + ax (upx - f0) + ay (upy - f0) runs on the FP32 pipe in hi + lo pairs
// (about 2^-46 relative per step) with one FP64 add to form the output. A thread owns one
// (i, j) column of the cell's slab and walks it along k, so the upwind choice, the CFL
// factors and the perimeter classification are worked out once per column.
constexpr int kConvThreads = 256;  // at most; launched as wide as column_threads says
constexpr int kConvAhead = 4;      // column nodes read ahead of the update

__global__ void __launch_bounds__(kConvThreads) k_convect2d(Convect2DArgs a) {
  const GridInfo& g = a.g;
  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny, NZ = g.nz;
  const int col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= NXY) return;
  const int cell = blockIdx.y;
  const int cx = cell % a.nxs, cy = cell / a.nxs;
  const int j = col / NX, i = col - j * NX;
  const double* f0p = a.f + static_cast<size_t>(cell) * nv + col;
  double* out = a.fconv + static_cast<size_t>(cell) * nv + col;
  const size_t row = static_cast<size_t>(a.nxs) * nv;
  const bool perim = (cx == 0 || cy == 0 || cx == a.nxs - 1 || cy == a.nys - 1);
  // upwind sources along x and y: a pointer to the column in the neighbour cell or a
  // wall ghost, or none
  const double* px = nullptr;
  const double* py = nullptr;
  bool hx = true, hy = true, zero = false;
  if (!perim) {
    px = (g.x[i] < 0.0) ? f0p + nv : f0p - nv;
    py = (g.y[j] < 0.0) ? f0p + row : f0p - row;
  } else {
    const int ci = axis_class(i, g.i_neg, g.i_pos, g.i_zero, g.i_zero_flag);
    const int cj = axis_class(j, g.j_neg, g.j_pos, g.j_zero, g.j_zero_flag);
    if (ci == kClsNone || cj == kClsNone) {
      zero = true;
    } else {
      if (ci == kClsNeg) {  // upwind is the right neighbour / right wall ghost
        if (cx < a.nxs - 1) px = f0p + nv;
        else if (a.bc_right == DVM_BC2D_WALL) px = a.ghost + static_cast<size_t>(a.base[1] + cy) * nv + col;
        else if (a.bc_right == DVM_BC2D_COUETTE) px = a.f + static_cast<size_t>(a.nxs) * cy * nv + col;
      } else if (ci == kClsPos) {  // left neighbour / left wall ghost
        if (cx > 0) px = f0p - nv;
        else if (a.bc_left == DVM_BC2D_WALL) px = a.ghost + static_cast<size_t>(a.base[0] + cy) * nv + col;
        else if (a.bc_left == DVM_BC2D_COUETTE) px = f0p;
      }
      if (cj == kClsNeg) {  // top neighbour / top wall ghost
        if (cy < a.nys - 1) py = f0p + row;
        else py = a.ghost + static_cast<size_t>(a.base[3] + cx) * nv + col;
      } else if (cj == kClsPos) {  // bottom neighbour / bottom wall ghost
        if (cy > 0) py = f0p - row;
        else py = a.ghost + static_cast<size_t>(a.base[2] + cx) * nv + col;
      }
      hx = (ci != kClsZero);
      hy = (cj != kClsZero);
    }
  }
  if (zero) {
    for (int k = 0; k < NZ; ++k) out[static_cast<size_t>(NXY) * k] = 0.0;
    return;
  }
  const float2 cxf = __ldg(a.cfl + i), cyf = __ldg(a.cfl + NX + j);
  const dfl AX = dfl_make(cxf.x, cxf.y), AY = dfl_make(cyf.x, cyf.y);
  if (hx && hy && px && py) {
    // both upwind sources present (every interior column): no per-node tests; the three
    // values of the next kConvAhead nodes are read while these are formed, so every thread
    // keeps 3 kConvAhead loads in flight
    double b0[kConvAhead], bx[kConvAhead], by[kConvAhead];
#pragma unroll
    for (int u = 0; u < kConvAhead; ++u) {
      const size_t o = static_cast<size_t>(NXY) * u;
      b0[u] = (u < NZ) ? __ldg(f0p + o) : 0.0;
      bx[u] = (u < NZ) ? __ldg(px + o) : 0.0;
      by[u] = (u < NZ) ? __ldg(py + o) : 0.0;
    }
    for (int k0 = 0; k0 < NZ; k0 += kConvAhead) {
      double n0[kConvAhead], nx[kConvAhead], ny[kConvAhead];
#pragma unroll
      for (int u = 0; u < kConvAhead; ++u) {
        const int k = k0 + kConvAhead + u;
        const size_t o = static_cast<size_t>(NXY) * k;
        n0[u] = (k < NZ) ? __ldg(f0p + o) : 0.0;
        nx[u] = (k < NZ) ? __ldg(px + o) : 0.0;
        ny[u] = (k < NZ) ? __ldg(py + o) : 0.0;
      }
#pragma unroll
      for (int u = 0; u < kConvAhead; ++u) {
        const int k = k0 + u;
        if (k >= NZ) break;
        const dfl F0 = dfl_from_double(b0[u]);
        const dfl acc = dfl_add(dfl_add(F0, dfl_mul(AX, dfl_sub(dfl_from_double(bx[u]), F0))),
                                dfl_mul(AY, dfl_sub(dfl_from_double(by[u]), F0)));
        out[static_cast<size_t>(NXY) * k] = dfl_to_double_fast(acc);
      }
#pragma unroll
      for (int u = 0; u < kConvAhead; ++u) { b0[u] = n0[u]; bx[u] = nx[u]; by[u] = ny[u]; }
    }
    return;
  }
#pragma unroll 4
  for (int k = 0; k < NZ; ++k) {
    const size_t o = static_cast<size_t>(NXY) * k;
    const dfl F0 = dfl_from_double(f0p[o]);
    dfl acc = F0;
    // a missing source (closed wall without ghost) contributes a zero value, as in the
    // reference's zero-initialised neighbour
    if (hx) acc = dfl_add(acc, dfl_mul(AX, dfl_sub(px ? dfl_from_double(px[o]) : dfl_make(0.f, 0.f), F0)));
    if (hy) acc = dfl_add(acc, dfl_mul(AY, dfl_sub(py ? dfl_from_double(py[o]) : dfl_make(0.f, 0.f), F0)));
    out[o] = dfl_to_double_fast(acc);
  }
}

cudaError_t launch_convect2d(const Convect2DArgs& a, int ncells, cudaStream_t s) {
  // a cell's columns in equal CTAs of whole warps (576 columns: 3 x 192, not 4.5 x 128)
  const int threads = column_threads(a.g, kConvThreads);
  dim3 grid((a.g.nx * a.g.ny + threads - 1) / threads, ncells);
  k_convect2d<<<grid, threads, 0, s>>>(a);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// 1-D (grid_ref convection/convection.f90:111-256): interior cells upwind; the two end
// cells start as copies of f (phi_conv == phi at step start) for the end conditions.
__global__ void __launch_bounds__(256) k_convect1d(Convect1DArgs a) {
  const GridInfo& g = a.g;
  const int nv = g.nv;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nv) return;
  const int cell = blockIdx.y;  // row cell / nxs, position nx in it
  const int nx = cell % a.nxs;
  const size_t off = static_cast<size_t>(cell) * nv + l;
  const double p0 = a.f[off];
  if (nx == 0 || nx == a.nxs - 1) { a.fconv[off] = p0; return; }
  const int i = l % g.nx;
  const double xv = g.x[i];
  const double cfl = a.factor * xv;
  // p0 - cfl (p1 - p0) for xi < 0, p0 - cfl (p0 - p_{-1}) otherwise
  a.fconv[off] = (xv < 0.0) ? fma(-cfl, a.f[off + nv] - p0, p0) : fma(-cfl, p0 - a.f[off - nv], p0);
}

cudaError_t launch_convect1d(const Convect1DArgs& a, cudaStream_t s) {
  dim3 grid((a.g.nv + 255) / 256, a.nxs * a.rows);
  k_convect1d<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// End conditions (grid_ref conditions/boundary_conditions.f90:319-1000). The node-local
// ones (specular, inflow Maxwellian, zero gradient) run one thread per node over both
// ends of every row (blockIdx.y = 2 row + end); the diffuse wall, which needs the incoming
// and outgoing flux sums of its end first, runs one CTA per end.
__global__ void __launch_bounds__(256) k_bc1d_nodes(Convect1DArgs a) {
  const GridInfo& g = a.g;
  const int e = blockIdx.y & 1;  // 0 left, 1 right
  const int row0 = (blockIdx.y >> 1) * a.nxs;
  const int bc = a.bc[e];
  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nv) return;
  const int nx = row0 + ((e == 0) ? 0 : a.nxs - 1);
  const double* f = a.f + static_cast<size_t>(nx) * nv;
  double* fc = a.fconv + static_cast<size_t>(nx) * nv;
  const double* W = a.wall[e];
  if (bc == DVM_BC1D_SPECULAR) {  // apply_specular_wall :446-564
    const double xv = g.x[l % NX];
    const double fac = a.factor * xv;
    if (e == 0 && xv < 0.0) fc[l] = f[l] - fac * (f[l + nv] - f[l]);
    if (e == 1 && xv > 0.0) fc[l] = f[l] - fac * (f[l] - f[l - nv]);
  } else if (bc == DVM_BC1D_INOUT) {  // apply_fixed_in_out_flow :783-913
    const double dens = W[DVM_WP_DENS], T = W[DVM_WP_TEMP], u = W[DVM_WP_U];
    const double mc = dens * maxwell_coeff(a.mass, T, a.pi);
    const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
    const double b3 = g.bx[i] * g.by[j] * g.bz[k];
    fc[l] = maxwellian(g.x[i], g.y[j], g.z[k], mc, a.mass, u, 0.0, 0.0, T) * b3;
  } else if (bc == DVM_BC1D_ZEROGRAD) {  // apply_zero_gradient_flow :915-962
    const double* src = a.fconv + static_cast<size_t>(row0 + (e == 0 ? 1 : a.nxs - 2)) * nv;
    fc[l] = src[l];
  }
}

cudaError_t launch_bc1d_nodes(const Convect1DArgs& a, cudaStream_t s) {
  dim3 grid((a.g.nv + 255) / 256, 2 * a.rows);
  k_bc1d_nodes<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

constexpr int kBc1dThreads = 1024;

__global__ void __launch_bounds__(kBc1dThreads) k_bc1d(Convect1DArgs a) {
  __shared__ double s_red[2 * 32];
  const GridInfo& g = a.g;
  const int e = blockIdx.x & 1;  // 0 left, 1 right
  const int row0 = (blockIdx.x >> 1) * a.nxs;
  const int nx = row0 + ((e == 0) ? 0 : a.nxs - 1);
  const int bc = a.bc[e];
  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const double* f = a.f + static_cast<size_t>(nx) * nv;
  double* fc = a.fconv + static_cast<size_t>(nx) * nv;
  const double* W = a.wall[e];
  if (bc == DVM_BC1D_DIFFUSE) {  // apply_diffuse_reflection :566-781
    const double T = W[DVM_WP_TEMP], u = W[DVM_WP_U], v = W[DVM_WP_V], w = W[DVM_WP_W];
    const double* f2 = a.f + static_cast<size_t>(row0 + (e == 0 ? 1 : a.nxs - 2)) * nv;
    const double mc = maxwell_coeff(a.mass, T, a.pi);
    double acc2[2] = {0.0, 0.0};  // incoming density, computed outgoing density
    for (int l = threadIdx.x; l < nv; l += blockDim.x) {
      const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
      const bool inc = (e == 0) ? (i <= g.i_neg) : (i >= g.i_pos);
      const bool out = (e == 0) ? (i >= g.i_pos) : (i <= g.i_neg);
      if (inc) acc2[0] += f[l];
      double val = 0.0;
      if (out) {
        const double b3 = g.bx[i] * g.by[j] * g.bz[k];
        const double M = maxwellian(g.x[i], g.y[j], g.z[k], mc, a.mass, u, v, w, T);
        val = M * b3;
        acc2[1] += M * b3;
      }
      fc[l] = val;
    }
    block_sum<2>(acc2, s_red);
    const double ratio = (a.acc * acc2[0]) / acc2[1];
    for (int l = threadIdx.x; l < nv; l += blockDim.x) fc[l] = ratio * fc[l];
    __syncthreads();
    // incoming half: upwind finite difference (overwrites)
    for (int l = threadIdx.x; l < nv; l += blockDim.x) {
      const int i = l % NX;
      const bool inc = (e == 0) ? (i <= g.i_neg) : (i >= g.i_pos);
      if (inc) {
        const double fac = a.factor * g.x[i];
        fc[l] = f[l] - fabs(fac) * (f[l] - f2[l]);
      }
    }
    __syncthreads();
    // specular remap of each incoming node; the reference interleaves the overwrite above
    // with these adds in loop order, so an add into an incoming node survives only when
    // that node comes no later than its source in the loop.
    if (a.acc < 1.0) {
      for (int l = threadIdx.x; l < nv; l += blockDim.x) {
        const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
        const bool inc = (e == 0) ? (i <= g.i_neg) : (i >= g.i_pos);
        if (!inc) continue;
        const double d = (1.0 - a.acc) * f[l];
        Stencil s;
        const int rb = remap(g, g.x, g.y, g.z, -g.x[i], g.y[j], g.z[k], 1.0, s);
        if (rb & 2) { atomicOr(a.err, DVM_EW_REMAP); continue; }
#pragma unroll
        for (int q = 0; q < 7; ++q) {
          const int n = s.node[q];
          if (n < 0) continue;
          const int ni = n % NX;
          const bool ninc = (e == 0) ? (ni <= g.i_neg) : (ni >= g.i_pos);
          if (ninc && n > l) continue;
          atomicAdd(fc + n, d * s.mass[q]);
        }
      }
    }
  }
}

cudaError_t launch_bc1d(const Convect1DArgs& a, cudaStream_t s) {
  k_bc1d<<<2 * a.rows, kBc1dThreads, 0, s>>>(a);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// k_moments: one CTA per cell; calculate_physical_properties (dist_funcs/physical_props.f90:
// 285-485, kernels :879-1087), compute_avg_speed (:1459-1507), compute_heat_flux
// (:1914-1986), compute_viscous_stress (:1988-2071).
//
// The reference makes separate passes over the cell for n, u, v, w, speed, then T, q, tau
// about u. Here one pass reduces along the k axis first: for every (i, j) column,
// G_p = sum_k f z'^p (p = 0..3, z' = z - w0), then the raw moments up to third order
// about the previous step's velocity (u0, v0, w0) follow from the columns with x' = x - u0,
// y' = y - v0, and the central moments by shifting to the new velocity; being taken about
// a velocity already close to u, the shift cancels nothing significant. The sums run on
// the FP32 pipe in hi + lo pairs (dfloat.cuh): each f and |xi| enters by an exact integer
// split, each product and sum carries its rounding error, so a thread's partial sums keep
// about 47 bits; only the per-thread totals go back to FP64 for the block reduction.
constexpr int kMomThreads = 256;
constexpr int kMomAcc = 14;
constexpr int kMomAhead = 4;  // column nodes read ahead of the sums

// The moments of one cell; src.begin(col) opens an (i, j) column and src.raw(k) returns
// the value of its node k. With kSplit, the cell's columns are dealt over the
// CTAs of a thread-block cluster (few cells: more CTAs than cells fill the SMs); each CTA
// reduces its columns and the partial totals meet in the shared memory of the cluster's
// first CTA, which adds them in rank order and forms the properties.
constexpr int kMomSplitMax = 4;

template <bool kSplit, class Src, bool kMirror = false>
__device__ __forceinline__ void moments_of_cell(const MomentArgs& a, int cell, Src& src) {
  __shared__ float2 s_red[kMomAcc * 32];
  __shared__ dfl s_ax[4 * kMaxAxis];  // x', x'^2, y', y'^2
  __shared__ dfl s_z[3 * kMaxAxis];   // z', z'^2, z'^3
  const GridInfo& g = a.g;
  const int NX = g.nx, NXY = g.nx * g.ny, NZ = g.nz;
  double* P = a.props + static_cast<size_t>(cell) * DVM_NPROP;
  const double u0 = isfinite(P[DVM_P_U]) ? P[DVM_P_U] : 0.0;
  const double v0 = isfinite(P[DVM_P_V]) ? P[DVM_P_V] : 0.0;
  const double w0 = isfinite(P[DVM_P_W]) ? P[DVM_P_W] : 0.0;
  for (int t = threadIdx.x; t < NX; t += blockDim.x) {
    const double xx = g.x[t] - u0;
    s_ax[t] = dfl_from_double(xx);
    s_ax[kMaxAxis + t] = dfl_from_double(xx * xx);
  }
  for (int t = threadIdx.x; t < g.ny; t += blockDim.x) {
    const double yy = g.y[t] - v0;
    s_ax[2 * kMaxAxis + t] = dfl_from_double(yy);
    s_ax[3 * kMaxAxis + t] = dfl_from_double(yy * yy);
  }
  for (int t = threadIdx.x; t < NZ; t += blockDim.x) {
    const double zz = g.z[t] - w0;
    s_z[t] = dfl_from_double(zz);
    s_z[kMaxAxis + t] = dfl_from_double(zz * zz);
    s_z[2 * kMaxAxis + t] = dfl_from_double(zz * zz * zz);
  }
  __syncthreads();
  // accumulators: 0 n | 1-3 M_x M_y M_z | 4-9 M_xx M_yy M_zz M_xy M_xz M_yz |
  // 10-12 T3_x T3_y T3_z (sum f c'_i |c'|^2) | 13 speed
  dacc sacc[kMomAcc];
#pragma unroll
  for (int q = 0; q < kMomAcc; ++q) dacc_zero(sacc[q]);
  const float2* speed = g.speed;
  unsigned rank = 0, nrank = 1;
  if constexpr (kSplit) {
    rank = cooperative_groups::this_cluster().block_rank();
    nrank = cooperative_groups::this_cluster().num_blocks();
  }
  for (int col = threadIdx.x + static_cast<int>(rank * blockDim.x); col < NXY;
       col += static_cast<int>(nrank * blockDim.x)) {
    dacc G0, G1, G2, G3, S;
    dacc_zero(G0); dacc_zero(G1); dacc_zero(G2); dacc_zero(G3); dacc_zero(S);
    src.begin(col);
    // the column's values are read kMomAhead nodes ahead of the ones being summed, so that
    // every thread keeps that many loads in flight
    double fb[kMomAhead];
#pragma unroll
    for (int u = 0; u < kMomAhead; ++u) fb[u] = (u < NZ) ? src.raw(u) : 0.0;
    double* mir = kMirror ? a.mirror + static_cast<size_t>(cell) * g.nv + col : nullptr;
    for (int k0 = 0; k0 < NZ; k0 += kMomAhead) {
      double fn[kMomAhead];
#pragma unroll
      for (int u = 0; u < kMomAhead; ++u)
        fn[u] = (k0 + kMomAhead + u < NZ) ? src.raw(k0 + kMomAhead + u) : 0.0;
#pragma unroll
      for (int u = 0; u < kMomAhead; ++u) {
        const int k = k0 + u;
        if (k >= NZ) break;
        if constexpr (kMirror) mir[NXY * k] = fb[u];
        const dfl fv = dfl_from_double(fb[u]);
        dacc_add(G0, fv);
        dacc_fma(G1, fv, s_z[k]);
        dacc_fma(G2, fv, s_z[kMaxAxis + k]);
        dacc_fma(G3, fv, s_z[2 * kMaxAxis + k]);
        const float2 sp = __ldg(speed + col + NXY * k);
        dacc_fma(S, fv, dfl_make(sp.x, sp.y));
      }
#pragma unroll
      for (int u = 0; u < kMomAhead; ++u) fb[u] = fn[u];
    }
    const int j = col / NX, i = col - j * NX;
    const dfl X = s_ax[i], X2 = s_ax[kMaxAxis + i];
    const dfl Y = s_ax[2 * kMaxAxis + j], Y2 = s_ax[3 * kMaxAxis + j];
    const dfl g0 = dfl_norm(G0.hi, G0.lo), g1 = dfl_norm(G1.hi, G1.lo);
    const dfl g2 = dfl_norm(G2.hi, G2.lo), g3 = dfl_norm(G3.hi, G3.lo);
    dacc_add(sacc[0], g0);
    dacc_fma(sacc[1], g0, X);
    dacc_fma(sacc[2], g0, Y);
    dacc_add(sacc[3], g1);
    dacc_fma(sacc[4], g0, X2);
    dacc_fma(sacc[5], g0, Y2);
    dacc_add(sacc[6], g2);
    dacc_fma(sacc[7], g0, dfl_mul(X, Y));
    dacc_fma(sacc[8], g1, X);
    dacc_fma(sacc[9], g1, Y);
    const dfl XY2 = dfl_add(X2, Y2);
    const dfl R2 = dfl_add(dfl_mul(XY2, g0), g2);   // sum_k f |c'|^2 over the column
    const dfl R2z = dfl_add(dfl_mul(XY2, g1), g3);  // sum_k f z' |c'|^2
    dacc_fma(sacc[10], R2, X);
    dacc_fma(sacc[11], R2, Y);
    dacc_add(sacc[12], R2z);
    dacc_add(sacc[13], dfl_norm(S.hi, S.lo));
  }
  double acc[kMomAcc];
  {
    __shared__ float2 s_sum[kMomAcc * kMomThreads];
    block_sum_dfl_t<kMomAcc>(sacc, s_sum, s_red, acc);
  }
  if constexpr (kSplit) {
    __shared__ double s_part[kMomSplitMax][kMomAcc];  // used in the cluster's first CTA
    cooperative_groups::cluster_group cl = cooperative_groups::this_cluster();
    if (threadIdx.x == 0) {
      double* dst = cl.map_shared_rank(&s_part[0][0], 0) + rank * kMomAcc;
#pragma unroll
      for (int q = 0; q < kMomAcc; ++q) dst[q] = acc[q];
    }
    cl.sync();  // also orders every CTA's reads of P before the first CTA writes it
    if (rank != 0) return;
    if (threadIdx.x == 0) {
#pragma unroll
      for (int q = 0; q < kMomAcc; ++q) {
        double t = s_part[0][q];
        for (unsigned r = 1; r < nrank; ++r) t += s_part[r][q];
        acc[q] = t;
      }
    }
  }
  if (threadIdx.x == 0) {
    // the previous moments, for the residual (only this thread writes P)
    const double n_old = P[DVM_P_DENS], t_old = P[DVM_P_TEMP];
    const double txx_old = P[DVM_P_TXX], tyy_old = P[DVM_P_TYY];
    const double txy_old = P[DVM_P_TXY], txz_old = P[DVM_P_TXZ], tyz_old = P[DVM_P_TYZ];
    const double n = acc[0];
    if (n == 0.0) {
      for (int q = 0; q < DVM_NPROP; ++q) P[q] = 0.0;
      return;  // (thread 0, after the block reduction)
    }
    const double m = a.mass;
    const double inv_n = 1.0 / n;  // one FP64 division for the per-density quotients
    const double dx = acc[1] * inv_n, dy = acc[2] * inv_n, dz = acc[3] * inv_n;
    const double d[3] = {dx, dy, dz};
    // central second moments C_ab = M_ab - n d_a d_b
    double C[3][3];
    C[0][0] = acc[4] - n * dx * dx; C[1][1] = acc[5] - n * dy * dy; C[2][2] = acc[6] - n * dz * dz;
    C[0][1] = C[1][0] = acc[7] - n * dx * dy;
    C[0][2] = C[2][0] = acc[8] - n * dx * dz;
    C[1][2] = C[2][1] = acc[9] - n * dy * dz;
    const double M1[3][3] = {{acc[4], acc[7], acc[8]}, {acc[7], acc[5], acc[9]},
                             {acc[8], acc[9], acc[6]}};
    const double S2 = acc[4] + acc[5] + acc[6];
    const double dd = dx * dx + dy * dy + dz * dz;
    double Q[3];
    for (int ii = 0; ii < 3; ++ii) {
      // sum f c_i |c|^2 with c = c' - d
      const double T3 = acc[10 + ii];
      const double mix = d[0] * M1[ii][0] + d[1] * M1[ii][1] + d[2] * M1[ii][2];
      Q[ii] = T3 - 2.0 * mix - d[ii] * S2 + 2.0 * n * d[ii] * dd;
    }
    const double t = 2.0 * m * (C[0][0] + C[1][1] + C[2][2]) * (inv_n * (1.0 / 3.0));
    const double p = 0.5 * n * t;
    P[DVM_P_DENS] = n;
    P[DVM_P_U] = u0 + dx; P[DVM_P_V] = v0 + dy; P[DVM_P_W] = w0 + dz;
    P[DVM_P_TEMP] = t;
    P[DVM_P_SPECIES_TEMP] = (3.0 * t + 0.0 * 0.0 + 0.0 * 0.0) / (3.0 + 0.0 + 0.0);
    P[DVM_P_AVG_SPEED] = acc[13] * inv_n;
    P[DVM_P_PRESSURE] = p;
    P[DVM_P_QX] = Q[0] * (0.5 * m); P[DVM_P_QY] = Q[1] * (0.5 * m); P[DVM_P_QZ] = Q[2] * (0.5 * m);
    P[DVM_P_TXX] = p - m * C[0][0]; P[DVM_P_TYY] = p - m * C[1][1]; P[DVM_P_TZZ] = p - m * C[2][2];
    P[DVM_P_TXY] = -m * C[0][1]; P[DVM_P_TXZ] = -m * C[0][2]; P[DVM_P_TYZ] = -m * C[1][2];
    for (int q = DVM_P_TYZ + 1; q < DVM_NPROP; ++q) P[q] = 0.0;
    uint32_t bad = 0;
    if (!isfinite(n) || !isfinite(t)) bad |= DVM_EW_NONFINITE;
    if (!(n > 0.0)) bad |= DVM_EW_NEGDENS;
    if (bad) atomicOr(a.err, bad);
    if (a.residual) {
      // relative change of n, u (on the thermal speed) and T since the last moments
      const double isu = 1.0 / (sqrt(fabs(t) / m) + 1e-300);
      double r = fabs(n - n_old) * fabs(inv_n);
      r = fmax(r, fabs(dx) * isu);
      r = fmax(r, fabs(dy) * isu);
      r = fmax(r, fabs(dz) * isu);
      r = fmax(r, fabs(t - t_old) / (fabs(t) + 1e-300));
      // and of the shear stresses on the pressure (the only moments a homogeneous
      // relaxation changes)
      const double ip = 1.0 / (fabs(p) + 1e-300);
      r = fmax(r, fabs(P[DVM_P_TXY] - txy_old) * ip);
      r = fmax(r, fabs(P[DVM_P_TXZ] - txz_old) * ip);
      r = fmax(r, fabs(P[DVM_P_TYZ] - tyz_old) * ip);
      r = fmax(r, fabs(P[DVM_P_TXX] - txx_old) * ip);
      r = fmax(r, fabs(P[DVM_P_TYY] - tyy_old) * ip);
      if (!(r >= 0.0)) r = 1e300;
      atomicMax(a.residual, static_cast<unsigned long long>(__double_as_longlong(r)));
    }
  }
}

// Node values straight from f.
struct MomSourceF {
  const double* f;
  int NXY, col;
  __device__ void begin(int c) { col = c; }
  __device__ double raw(int k) const { return __ldg(f + col + NXY * k); }
};

template <bool kMirror>
__global__ void __launch_bounds__(kMomThreads, 3) k_moments(MomentArgs a) {
  const int cell = blockIdx.x;
  MomSourceF src{a.f + static_cast<size_t>(cell) * a.g.nv, a.g.nx * a.g.ny, 0};
  moments_of_cell<false, MomSourceF, kMirror>(a, cell, src);
}

// Launched in clusters of 2 or 4 CTAs per cell.
template <bool kMirror>
__global__ void __launch_bounds__(kMomThreads, 3) k_moments_split(MomentArgs a) {
  const int cell = static_cast<int>(blockIdx.x / cooperative_groups::this_cluster().num_blocks());
  MomSourceF src{a.f + static_cast<size_t>(cell) * a.g.nv, a.g.nx * a.g.ny, 0};
  moments_of_cell<true, MomSourceF, kMirror>(a, cell, src);
}


cudaError_t launch_moments(const MomentArgs& a, cudaStream_t s) {
  // CTAs per cell: enough that a launch of few cells still covers the SMs twice over
  int split = 1;
  while (split < kMomSplitMax && a.ncells * split < 2 * sm_count()) split *= 2;
  const bool mirror = a.mirror != nullptr;
  if (split == 1) {
    if (mirror) k_moments<true><<<a.ncells, column_threads(a.g, kMomThreads), 0, s>>>(a);
    else k_moments<false><<<a.ncells, column_threads(a.g, kMomThreads), 0, s>>>(a);
    return cudaGetLastError();
  }
  GridInfo gs = a.g;  // the columns one CTA walks
  const int cols = a.g.nx * a.g.ny;
  gs.nx = (cols + split - 1) / split;
  gs.ny = 1;
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(static_cast<unsigned>(a.ncells * split));
  cfg.blockDim = dim3(static_cast<unsigned>(column_threads(gs, kMomThreads)));
  cfg.dynamicSmemBytes = 0;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeClusterDimension;
  attr[0].val.clusterDim.x = static_cast<unsigned>(split);
  attr[0].val.clusterDim.y = 1;
  attr[0].val.clusterDim.z = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return mirror ? cudaLaunchKernelEx(&cfg, k_moments_split<true>, a)
                : cudaLaunchKernelEx(&cfg, k_moments_split<false>, a);
}

// ----------------------------------------------------------------------------------------
__global__ void k_flush(double* buf, size_t n) {
  for (size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<size_t>(gridDim.x) * blockDim.x)
    buf[t] = static_cast<double>(t);
}

// End of a device-counted step: advance the Philox step counter and, when asked, add the
// step's sample total to a running count.
__global__ void k_step_end(uint32_t* counter, long long* acc, const long long* total) {
  *counter += 1u;
  if (acc && total) *acc += *total;
}

cudaError_t launch_step_end(uint32_t* counter, long long* acc, const long long* total,
                            cudaStream_t s) {
  k_step_end<<<1, 1, 0, s>>>(counter, acc, total);
  return cudaGetLastError();
}

// FP64 atomic-add throughput probe: every thread adds to pseudo-random doubles of a
// window of n (the scatter pattern of k_collide over an L2-resident slab of f).
__global__ void __launch_bounds__(256) k_atomic_probe(double* buf, size_t n, int per_thread) {
  uint32_t x = 0x9E3779B9u * (blockIdx.x * blockDim.x + threadIdx.x + 1u);
  for (int r = 0; r < per_thread; ++r) {
    x ^= x << 13; x ^= x >> 17; x ^= x << 5;
    atomicAdd(buf + (x % n), 1e-300);
  }
}

// Failure-path check: waits on a barrier that nothing completes, with the bounded wait the
// bulk-copy kernels use; the wait gives up and reports DVM_EW_WAIT in the error word.
__global__ void k_wait_selftest(uint32_t* err) {
  __shared__ __align__(8) uint64_t s_bar;
  if (threadIdx.x == 0) mbar_init(&s_bar, 1);
  __syncthreads();
  if (!mbar_wait(&s_bar, 0u) && threadIdx.x == 0) atomicOr(err, static_cast<uint32_t>(DVM_EW_WAIT));
  __syncthreads();
}

cudaError_t launch_wait_selftest(uint32_t* err, cudaStream_t s) {
  k_wait_selftest<<<1, 32, 0, s>>>(err);
  return cudaGetLastError();
}

cudaError_t launch_atomic_probe(double* buf, size_t n, int blocks, int per_thread,
                                cudaStream_t s) {
  k_atomic_probe<<<blocks, 256, 0, s>>>(buf, n, per_thread);
  return cudaGetLastError();
}

cudaError_t launch_flush(double* buf, size_t n, cudaStream_t s) {
  k_flush<<<1216, 256, 0, s>>>(buf, n);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// Grouped launches: one launch of each kernel advances every instance of a batch, whatever
// its velocity grid. Groups own consecutive CTAs; a CTA looks its group up in the launch
// parameters (first[g] <= blockIdx.x < first[g+1]) and runs that group's code path with
// the group's own arguments, so the instances of all grids share the SMs in one launch.
__device__ __forceinline__ int group_of(const int* first, int ngroups, int x) {
  int gi = 0;
  while (gi + 1 < ngroups && x >= first[gi + 1]) ++gi;
  return gi;
}

template <int T>
__global__ void __launch_bounds__(T, 1024 / T) k_cdf_grouped(const __grid_constant__ GroupedCdf m) {
  const int gi = group_of(m.first, m.ngroups, static_cast<int>(blockIdx.x));
  cdf_cta<T>(m.a[gi], static_cast<int>(blockIdx.x) - m.first[gi]);
}

template <int T>
static cudaError_t launch_cdf_grouped_t(const GroupedCdf& m, cudaStream_t s) {
  constexpr int smem = (T / 32) * kCdfTrWarp * static_cast<int>(sizeof(long long));
  const cudaError_t e =
      cudaFuncSetAttribute(k_cdf_grouped<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  if (e != cudaSuccess) return e;
  k_cdf_grouped<T><<<m.first[m.ngroups], T, smem, s>>>(m);
  return cudaGetLastError();
}

cudaError_t launch_cdf_grouped(const GroupedCdf& m, int cdf_threads, cudaStream_t s) {
  if (m.ngroups < 1 || m.ngroups > kMaxGroups || m.first[m.ngroups] < 1) return cudaErrorInvalidValue;
  if (cdf_threads >= 1024) return launch_cdf_grouped_t<1024>(m, s);
  if (cdf_threads >= 512) return launch_cdf_grouped_t<512>(m, s);
  return launch_cdf_grouped_t<256>(m, s);
}

__global__ void __launch_bounds__(1024) k_plan_grouped(const __grid_constant__ GroupedPlan m) {
  const int gi = static_cast<int>(blockIdx.x);
  plan_cta(m.ncells[gi], m.plan[gi], m.chunk_off[gi], m.total[gi], m.warps[gi]);
}

cudaError_t launch_plan_grouped(const GroupedPlan& m, cudaStream_t s) {
  if (m.ngroups < 1 || m.ngroups > kMaxGroups) return cudaErrorInvalidValue;
  k_plan_grouped<<<m.ngroups, 1024, 0, s>>>(m);
  return cudaGetLastError();
}

// Groups own consecutive CTAs (first[g] <= blockIdx.x < first[g+1]). Three CTAs per SM:
// the per-group arguments are read by index and need the registers that 80 per thread
// leave (at 64 the general FP64 kernel spills three times as much and runs 25 % slower;
// the common configuration's copies at four measured 9.04 against 7.96 ms (FP64) and
// 6.2 against 5.3 ms (FP32) per batch step). kFast when every group has the
// configuration of collide_fast.
template <bool kFast>
__global__ void __launch_bounds__(kCollideChunk, 3) k_collide_grouped(const __grid_constant__ GroupedCollide m) {
  const int b = static_cast<int>(blockIdx.x);
  const int gi = group_of(m.first, m.ngroups, b);
  collide_cta<kFast, false>(m.a[gi], b - m.first[gi], m.first[gi + 1] - m.first[gi]);
}

template <bool kFast>
__global__ void __launch_bounds__(kCollideChunk, 3) k_collide_f32_grouped(const __grid_constant__ GroupedCollide m) {
  const int b = static_cast<int>(blockIdx.x);
  const int gi = group_of(m.first, m.ngroups, b);
  collide_f32_cta<kFast, false>(m.a[gi], m.tf[gi], m.df[gi], b - m.first[gi], m.first[gi + 1] - m.first[gi]);
}

static bool grouped_fast(const GroupedCollide& m) {
  for (int gi = 0; gi < m.ngroups; ++gi)
    if (!collide_fast(m.a[gi])) return false;
  return true;
}

static const void* grouped_collide_fn(const GroupedCollide& m, bool fp32) {
  const bool fast = grouped_fast(m);
  if (fp32)
    return fast ? reinterpret_cast<const void*>(k_collide_f32_grouped<true>)
                : reinterpret_cast<const void*>(k_collide_f32_grouped<false>);
  return fast ? reinterpret_cast<const void*>(k_collide_grouped<true>)
              : reinterpret_cast<const void*>(k_collide_grouped<false>);
}

static size_t collide_grouped_smem(const GroupedCollide& m, bool fp32) {
  size_t smem = 0;
  for (int gi = 0; gi < m.ngroups; ++gi) {
    const size_t b = fp32 ? collide_f32_smem_layout(m.a[gi].g, m.a[gi].t, m.tf[gi].gtab_smem).total
                          : collide_smem_bytes(m.a[gi].g, m.a[gi].t);
    smem = b > smem ? b : smem;
  }
  return smem;
}

int collide_grouped_blocks_per_sm(const GroupedCollide& m, bool fp32) {
  const size_t smem = collide_grouped_smem(m, fp32);
  const void* fn = grouped_collide_fn(m, fp32);
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, fn, kCollideChunk, smem) != cudaSuccess)
    n = 1;
  cudaGetLastError();
  return n > 0 ? n : 1;
}

cudaError_t launch_collide_grouped(const GroupedCollide& m, bool fp32, cudaStream_t s) {
  if (m.ngroups < 1 || m.ngroups > kMaxGroups) return cudaErrorInvalidValue;
  if (m.first[0] != 0) return cudaErrorInvalidValue;
  for (int gi = 0; gi < m.ngroups; ++gi)
    if (m.first[gi + 1] <= m.first[gi]) return cudaErrorInvalidValue;  // every group owns a CTA
  const size_t smem = collide_grouped_smem(m, fp32);
  const void* fn = grouped_collide_fn(m, fp32);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  const unsigned grid = static_cast<unsigned>(m.first[m.ngroups]);
  const bool fast = grouped_fast(m);
  if (fp32) {
    if (fast) k_collide_f32_grouped<true><<<grid, kCollideChunk, smem, s>>>(m);
    else k_collide_f32_grouped<false><<<grid, kCollideChunk, smem, s>>>(m);
  } else {
    if (fast) k_collide_grouped<true><<<grid, kCollideChunk, smem, s>>>(m);
    else k_collide_grouped<false><<<grid, kCollideChunk, smem, s>>>(m);
  }
  return cudaGetLastError();
}

__global__ void __launch_bounds__(kProjThreads, 3) k_project_grouped(const __grid_constant__ GroupedProject m) {
  const int gi = group_of(m.first, m.ngroups, static_cast<int>(blockIdx.x));
  const ProjectArgs& a = m.a[gi];
  const int cell = static_cast<int>(blockIdx.x) - m.first[gi];
  const size_t off = static_cast<size_t>(cell) * a.g.nv;
  project_cell(a.g, a.df + off, true, a.f + off, a.props + static_cast<size_t>(cell) * DVM_NPROP);
}

cudaError_t launch_project_grouped(const GroupedProject& m, cudaStream_t s) {
  if (m.ngroups < 1 || m.ngroups > kMaxGroups || m.first[m.ngroups] < 1) return cudaErrorInvalidValue;
  int threads = 32;
  for (int gi = 0; gi < m.ngroups; ++gi) {
    const int t = column_threads(m.a[gi].g, kProjThreads);
    threads = t > threads ? t : threads;
  }
  k_project_grouped<<<m.first[m.ngroups], threads, 0, s>>>(m);
  return cudaGetLastError();
}

__global__ void __launch_bounds__(kMomThreads, 3) k_moments_grouped(const __grid_constant__ GroupedMoments m) {
  const int gi = group_of(m.first, m.ngroups, static_cast<int>(blockIdx.x));
  const MomentArgs& a = m.a[gi];
  const int cell = static_cast<int>(blockIdx.x) - m.first[gi];
  MomSourceF src{a.f + static_cast<size_t>(cell) * a.g.nv, a.g.nx * a.g.ny, 0};
  moments_of_cell<false>(a, cell, src);
}

cudaError_t launch_moments_grouped(const GroupedMoments& m, cudaStream_t s) {
  if (m.ngroups < 1 || m.ngroups > kMaxGroups || m.first[m.ngroups] < 1) return cudaErrorInvalidValue;
  int threads = 32;
  for (int gi = 0; gi < m.ngroups; ++gi) {
    const int t = column_threads(m.a[gi].g, kMomThreads);
    threads = t > threads ? t : threads;
  }
  k_moments_grouped<<<m.first[m.ngroups], threads, 0, s>>>(m);
  return cudaGetLastError();
}

}  // namespace dvm

