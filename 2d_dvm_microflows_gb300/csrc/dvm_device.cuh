// dvm_device.cuh -- device helpers shared by the DVM kernels (sm_103a).
//
// Each helper restates one reference routine (aarthisekaran11/2D_DVM_microflows,
// software/trunk/src) with the same operation order, so FP64 results agree with the
// Fortran to rounding. Discrete decisions (nearest node, stencil signs, bucket choice)
// are taken on the same quantities as the reference.
#pragma once
#include <cstdint>
#include <cmath>

#include "../../include/dvm_gpu.h"

namespace dvm {

constexpr double kPiReference = 3.1459265358979323;  // utils/constants.f90:30 (sic)
constexpr double kPiExact = 3.14159265358979323846;
constexpr double kDoubleTol = 1.0e-13;               // utils/constants.f90:52
constexpr int kNRef = 1000;                          // variance_reduction.f90:471-493
constexpr int kMaxSearchIters = 256;
constexpr int kMaxAxis = 128;                        // nodes per velocity axis
constexpr int kMaxRepl = 16;

// Velocity grid metadata derived once by dvm_create (grid/velocity_grid.f90:271-726).
struct GridInfo {
  int nx, ny, nz, nv;
  double xv_min, yv_min, zv_min;
  double xv_factor, yv_factor, zv_factor;
  int i_zero, i_neg, i_pos, j_zero, j_neg, j_pos;
  int i_zero_flag, j_zero_flag;
  double beta3_min;
  const double* x;   // device arrays
  const double* y;
  const double* z;
  const double* bx;
  const double* by;
  const double* bz;
  const float2* speed;  // |xi| per node as a hi + lo pair (moments); may be null where unused
};

// ----------------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al., SC'11). Counter = (sample, cell, step, sub | call << 2),
// key = seed. Every sample owns its counter, so a skipped sample consumes nothing and the
// stream does not depend on launch shape.
__device__ __forceinline__ void philox4x32_10(uint32_t c0, uint32_t c1, uint32_t c2, uint32_t c3,
                                              uint32_t k0, uint32_t k1, uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = static_cast<uint64_t>(0xD2511F53u) * c0;
    const uint64_t p1 = static_cast<uint64_t>(0xCD9E8D57u) * c2;
    const uint32_t n0 = static_cast<uint32_t>(p1 >> 32) ^ c1 ^ k0;
    const uint32_t n2 = static_cast<uint32_t>(p0 >> 32) ^ c3 ^ k1;
    c0 = n0; c1 = static_cast<uint32_t>(p1); c2 = n2; c3 = static_cast<uint32_t>(p0);
    k0 += 0x9E3779B9u;
    k1 += 0xBB67AE85u;
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// philox4x32_10 with the key schedule given: rk[2 r], rk[2 r + 1] are the keys of round r
// (k0 + r 0x9E3779B9, k1 + r 0xBB67AE85), formed once on the host; kernels that hold rk
// in their launch parameters read each key as an operand instead of adding it up.
__device__ __forceinline__ void philox4x32_10_rk(uint32_t c0, uint32_t c1, uint32_t c2,
                                                 uint32_t c3, const uint32_t (&rk)[20],
                                                 uint32_t out[4]) {
#pragma unroll
  for (int r = 0; r < 10; ++r) {
    const uint64_t p0 = static_cast<uint64_t>(0xD2511F53u) * c0;
    const uint64_t p1 = static_cast<uint64_t>(0xCD9E8D57u) * c2;
    const uint32_t n0 = static_cast<uint32_t>(p1 >> 32) ^ c1 ^ rk[2 * r];
    const uint32_t n2 = static_cast<uint32_t>(p0 >> 32) ^ c3 ^ rk[2 * r + 1];
    c0 = n0; c1 = static_cast<uint32_t>(p1); c2 = n2; c3 = static_cast<uint32_t>(p0);
  }
  out[0] = c0; out[1] = c1; out[2] = c2; out[3] = c3;
}

// The key schedule of a seed (k0, k1 = its low and high words).
__host__ __device__ inline void philox_key_schedule(uint64_t seed, uint32_t (&rk)[20]) {
  for (int r = 0; r < 10; ++r) {
    rk[2 * r] = static_cast<uint32_t>(seed) + static_cast<uint32_t>(r) * 0x9E3779B9u;
    rk[2 * r + 1] = static_cast<uint32_t>(seed >> 32) + static_cast<uint32_t>(r) * 0xBB67AE85u;
  }
}

// m 2^-53 for a 53-bit integer m, built from the bits (exact; no FP64 op).
__device__ __forceinline__ double u53m(uint64_t m) {
  if (m == 0) return 0.0;
  const int p = 63 - __clzll(static_cast<long long>(m));  // top bit, 0..52
  const uint64_t mant = (m << (52 - p)) & ((1ull << 52) - 1);
  return __longlong_as_double(static_cast<long long>((static_cast<uint64_t>(p + 970) << 52) | mant));
}

// m 2^-53 from the top 53 bits of (hi, lo).
__device__ __forceinline__ double u53(uint32_t lo, uint32_t hi) {
  return u53m(((static_cast<uint64_t>(hi) << 32) | lo) >> 11);
}

// The two 53-bit integers m behind philox_uniform2's uniforms (u = m 2^-53), for callers
// that work on the integers directly.
__device__ __forceinline__ void philox_u53x2(uint64_t seed, uint32_t sample, uint32_t cell,
                                             uint32_t step, uint32_t sub, uint32_t call,
                                             unsigned long long& m0, unsigned long long& m1) {
  uint32_t o[4];
  philox4x32_10(sample, cell, step, (sub & 3u) | (call << 2), static_cast<uint32_t>(seed),
                static_cast<uint32_t>(seed >> 32), o);
  m0 = ((static_cast<uint64_t>(o[1]) << 32) | o[0]) >> 11;
  m1 = ((static_cast<uint64_t>(o[3]) << 32) | o[2]) >> 11;
}

// philox_u53x2 from a key schedule.
__device__ __forceinline__ void philox_u53x2_rk(const uint32_t (&rk)[20], uint32_t sample,
                                                uint32_t cell, uint32_t step, uint32_t sub,
                                                uint32_t call, unsigned long long& m0,
                                                unsigned long long& m1) {
  uint32_t o[4];
  philox4x32_10_rk(sample, cell, step, (sub & 3u) | (call << 2), rk, o);
  m0 = ((static_cast<uint64_t>(o[1]) << 32) | o[0]) >> 11;
  m1 = ((static_cast<uint64_t>(o[3]) << 32) | o[2]) >> 11;
}

// An out-of-line copy of philox_u53x2_rk, for a kernel that draws from two places in its
// sample loop: one copy of the ten rounds in its code instead of two inlined ones (the
// FP64 collide kernel waits on instruction fetch otherwise).
static __device__ __noinline__ void philox_u53x2_rk_call(const uint32_t (&rk)[20],
                                                         uint32_t sample, uint32_t cell,
                                                         uint32_t step, uint32_t sub,
                                                         uint32_t call, unsigned long long& m0,
                                                         unsigned long long& m1) {
  philox_u53x2_rk(rk, sample, cell, step, sub, call, m0, m1);
}

// u < kDoubleTol for u = m 2^-53 exactly when m < kTolU53 = ceil(kDoubleTol 2^53).
constexpr double kTolScaled = kDoubleTol * 9007199254740992.0;
constexpr unsigned long long kTolU53 =
    static_cast<double>(static_cast<unsigned long long>(kTolScaled)) < kTolScaled
        ? static_cast<unsigned long long>(kTolScaled) + 1
        : static_cast<unsigned long long>(kTolScaled);

__device__ __forceinline__ void philox_uniform2(uint64_t seed, uint32_t sample, uint32_t cell,
                                                uint32_t step, uint32_t sub, uint32_t call,
                                                double& u0, double& u1) {
  uint32_t o[4];
  philox4x32_10(sample, cell, step, (sub & 3u) | (call << 2), static_cast<uint32_t>(seed),
                static_cast<uint32_t>(seed >> 32), o);
  u0 = u53(o[0], o[1]);
  u1 = u53(o[2], o[3]);
}

// ----------------------------------------------------------------------------------------
// utils/math_utils.f90:38-60 and Fortran SIGN(1, i)
__device__ __forceinline__ int isgn(double x) { return signbit(x) ? -1 : 1; }
__device__ __forceinline__ double dsgn(double x) { return signbit(x) ? -1.0 : 1.0; }
__device__ __forceinline__ int isign1(int i) { return i < 0 ? -1 : 1; }

// compute_maxwellian, dist_funcs/dist_func.f90:317-344
__device__ __forceinline__ double maxwellian(double x, double y, double z, double coeff,
                                             double mass, double u, double v, double w,
                                             double temp) {
  double cx = x - u; cx = cx * cx;
  double cy = y - v; cy = cy * cy;
  double cz = z - w; cz = cz * cz;
  const double csq = cx + cy + cz;
  return coeff * exp(-csq * mass / temp);
}

__host__ __device__ inline double maxwell_coeff(double mass, double temp, double pi) {
  return sqrt(mass * mass * mass / (pi * pi * pi * temp * temp * temp));
}

// ----------------------------------------------------------------------------------------
// binary_search_with_first_guess, utils/sort_and_search.f90:130-183. Returns 0 on success.
__device__ __forceinline__ int bsearch_first_guess(int& index, double val, const double* arr,
                                                   int mn, int mx) {
  if (arr[mn] > val) { index = mn; return 0; }
  if (arr[mx] < val) { index = mx; return 0; }
  int left = mn, right = mx;
  int idx = index;
  if (idx < mn || idx > mx) { index = mn; return 1; }
  if (fabs(val - arr[idx]) < kDoubleTol) return 0;
  if (idx == right) idx = idx - 1;
  for (int it = 0; it < kMaxSearchIters; ++it) {
    const double a0 = arr[idx], a1 = arr[idx + 1];
    if (val > a0 && val <= a1) {
      if (fabs(val - a0) > fabs(val - a1)) idx = idx + 1;
      index = idx;
      return 0;
    }
    if (val > a0) left = idx; else right = idx;
    idx = left + (right - left) / 2;
  }
  index = idx;
  return 1;
}

// find_boundary_stencil, collisions/remapping.f90:396-438
__device__ __forceinline__ void find_boundary_stencil(int& sa, int& sb, int& sc, double abc,
                                                      int oi, int oj, int ok, const double* x,
                                                      const double* y, const double* z,
                                                      int i_min, int i_max, int j_min,
                                                      int j_max, int k_min, int k_max) {
  while (oi + sa > i_min && oi + sa < i_max) {
    if (fabs(abc) > 0.5 * fabs(x[oi + sa] - x[oi])) sa = sa + isign1(sa);
    else break;
  }
  while (oj + sb > j_min && oj + sb < j_max && oj - sb > j_min && oj - sb < j_max) {
    if (fabs(abc) > 0.5 * fabs(y[oj + sb] - y[oj])) sb = sb + isign1(sb);
    else break;
  }
  while (ok + sc > k_min && ok + sc < k_max && ok - sc > k_min && ok - sc < k_max) {
    if (fabs(abc) > 0.5 * fabs(z[ok + sc] - z[ok])) sc = sc + isign1(sc);
    else break;
  }
}

// Result of compute_remapping_quantities: stencil nodes as linear indices (-1 = unused)
// and their weights.
struct Stencil {
  int node[7];
  double mass[7];
};

// compute_remapping_quantities, collisions/remapping.f90:92-394, non-uniform branch (the
// reference forces uniform_grid = .false. at :121-122). x/y/z may live in shared memory.
// Returns 0, bit 0 = a search gave up, bit 1 = no exterior node (reference stops, :345).
__device__ __forceinline__ int remap(const GridInfo& g, const double* x, const double* y,
                                     const double* z, double u, double v, double w,
                                     double f_off, Stencil& s) {
  const int i_min = 0, i_max = g.nx - 1, j_min = 0, j_max = g.ny - 1, k_min = 0,
            k_max = g.nz - 1;
  int corner = 0, bad = 0;
  int o_i = static_cast<int>(llround(g.xv_factor * (u - g.xv_min)));
  bad |= bsearch_first_guess(o_i, u, x, i_min, i_max);
  if (o_i >= i_max) { o_i = i_max; corner++; }
  else if (o_i <= i_min) { o_i = i_min; corner++; }
  int o_j = static_cast<int>(llround(g.yv_factor * (v - g.yv_min)));
  bad |= bsearch_first_guess(o_j, v, y, j_min, j_max);
  if (o_j >= j_max) { o_j = j_max; corner++; }
  else if (o_j <= j_min) { o_j = j_min; corner++; }
  int o_k = static_cast<int>(llround(g.zv_factor * (w - g.zv_min)));
  bad |= bsearch_first_guess(o_k, w, z, k_min, k_max);
  if (o_k >= k_max) { o_k = k_max; corner++; }
  else if (o_k <= k_min) { o_k = k_min; corner++; }
  if (corner == 3) {
    o_i -= isign1(o_i - (i_min + 1));
    o_j -= isign1(o_j - (j_min + 1));
    o_k -= isign1(o_k - (k_min + 1));
  }
  const double ox = x[o_i], oy = y[o_j], oz = z[o_k];
  const double a = u - ox, b = v - oy, c = w - oz;
  int sa = isgn(a), sb = isgn(b), sc = isgn(c);
  if (o_i + sa > i_max || o_i + sa < i_min) {
    sa = -1 * sa;
    find_boundary_stencil(sa, sb, sc, a, o_i, o_j, o_k, x, y, z, i_min, i_max, j_min, j_max,
                          k_min, k_max);
  }
  if (o_j + sb > j_max || o_j + sb < j_min) {
    sb = -1 * sb;
    find_boundary_stencil(sb, sa, sc, b, o_j, o_i, o_k, y, x, z, j_min, j_max, i_min, i_max,
                          k_min, k_max);
  }
  if (o_k + sc > k_max || o_k + sc < k_min) {
    sc = -1 * sc;
    find_boundary_stencil(sc, sb, sa, c, o_k, o_j, o_i, z, y, x, k_min, k_max, j_min, j_max,
                          i_min, i_max);
  }
  const double int_x = x[o_i + sa] - ox;
  const double int_y = y[o_j + sb] - oy;
  const double int_z = z[o_k + sc] - oz;
  int fx = 0, fy = 0, fz = 0;
  double ext_x = 0.0, ext_y = 0.0, ext_z = 0.0;
  if (o_i - sa <= i_max && o_i - sa >= i_min) { fx = 1; ext_x = x[o_i - sa] - ox; }
  if (o_j - sb <= j_max && o_j - sb >= j_min) { fy = 2; ext_y = y[o_j - sb] - oy; }
  if (o_k - sc <= k_max && o_k - sc >= k_min) { fz = 4; ext_z = z[o_k - sc] - oz; }
  const int flag = fx + fy + fz;
  const double num = f_off * (a * a + b * b + c * c - a * int_x - b * int_y - c * int_z);
  double den = 0.0;
  if (fx) den = ext_x * (ext_x - int_x);
  if (fy) den = den + ext_y * (ext_y - int_y);
  if (fz) den = den + ext_z * (ext_z - int_z);
  double f_e = 0.0;
  if (flag == 0) bad |= 2;
  else f_e = num / den;
  const double f_ex = fx ? f_e : 0.0, f_ey = fy ? f_e : 0.0, f_ez = fz ? f_e : 0.0;
  const double f_ix = (f_off * a - f_ex * ext_x) / int_x;
  const double f_iy = (f_off * b - f_ey * ext_y) / int_y;
  const double f_iz = (f_off * c - f_ez * ext_z) / int_z;
  const double f_o = f_off - f_ix - f_iy - f_iz - f_ex - f_ey - f_ez;
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

// ----------------------------------------------------------------------------------------
// referenced_search, utils/sort_and_search.f90:40-86 (0-based node). The bucket table is
// ref[2*(bucket-1) + {0,1}]. Where the reference's loop would not terminate (the target
// outside the bucket bounds by a rounding), a search of the whole CDF takes over and the
// error word records it.
__device__ __forceinline__ int referenced_search(const double* __restrict__ cum,
                                                 const int2* __restrict__ ref, int n, double R,
                                                 uint32_t& bad) {
  if (R < kDoubleTol) return 0;
  int i = static_cast<int>(ceil(R * 1000.0));
  i = i < 1 ? 1 : (i > kNRef ? kNRef : i);
  const int2 lr = ref[i - 1];
  int left = lr.x, right = lr.y;
  int idx = left + (right - left) / 2;
  if (left == right) return idx < n ? idx : n - 1;
  const double adj = R * cum[n];
  for (int it = 0; it < kMaxSearchIters; ++it) {
    if (idx < 0 || idx >= n) break;
    const double c0 = cum[idx];
    if (adj > c0 && adj <= cum[idx + 1]) return idx;
    if (adj > c0) left = idx; else right = idx;
    idx = left + (right - left) / 2;
  }
  bad |= DVM_EW_SEARCH;
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = lo + (hi - lo) / 2;
    if (adj > cum[mid]) lo = mid; else hi = mid;
  }
  return lo;
}

// ----------------------------------------------------------------------------------------
// Block-wide reductions and scans (NT threads, NT a multiple of 32, NT <= 1024).
__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// Sums NV values per thread across the block; result broadcast to every thread.
// s_red must hold NV*32 doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double* s_red) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = warp_sum(v[q]);
  if (lane == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) s_red[q * 32 + warp] = v[q];
  }
  __syncthreads();
  if (warp == 0) {
#pragma unroll
    for (int q = 0; q < NV; ++q) {
      double t = lane < nw ? s_red[q * 32 + lane] : 0.0;
      t = warp_sum(t);
      if (lane == 0) s_red[q * 32] = t;
    }
  }
  __syncthreads();
#pragma unroll
  for (int q = 0; q < NV; ++q) v[q] = s_red[q * 32];
  __syncthreads();
}

// Inclusive scan of two doubles per thread across the block; tot gets the block totals.
// s_scan must hold 64 doubles.
__device__ __forceinline__ void block_scan2(double& a, double& b, double& tot_a, double& tot_b,
                                            double* s_scan) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const double ta = __shfl_up_sync(0xffffffffu, a, o);
    const double tb = __shfl_up_sync(0xffffffffu, b, o);
    if (lane >= o) { a += ta; b += tb; }
  }
  if (lane == 31) { s_scan[warp] = a; s_scan[32 + warp] = b; }
  __syncthreads();
  if (warp == 0) {
    double wa = lane < nw ? s_scan[lane] : 0.0;
    double wb = lane < nw ? s_scan[32 + lane] : 0.0;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const double ta = __shfl_up_sync(0xffffffffu, wa, o);
      const double tb = __shfl_up_sync(0xffffffffu, wb, o);
      if (lane >= o) { wa += ta; wb += tb; }
    }
    s_scan[lane] = wa;
    s_scan[32 + lane] = wb;
  }
  __syncthreads();
  if (warp > 0) { a += s_scan[warp - 1]; b += s_scan[32 + warp - 1]; }
  tot_a = s_scan[nw - 1];
  tot_b = s_scan[32 + nw - 1];
  __syncthreads();
}

// ----------------------------------------------------------------------------------------
// Bulk global->shared copies on the async proxy (cp.async.bulk) completed through an
// mbarrier transaction count, and a bounded wait on the barrier phase.
__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(bar)), "r"(count)
               : "memory");
}

// Makes barrier initialisation and earlier generic-proxy accesses of shared memory visible
// to the async proxy.
__device__ __forceinline__ void fence_proxy_async() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// One thread: expect `bytes` on bar and start the copy of `bytes` (a multiple of 16, both
// addresses 16-byte aligned) from global src to shared dst.
__device__ __forceinline__ void bulk_load(void* dst, const void* src, uint32_t bytes,
                                          uint64_t* bar) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(bar)),
               "r"(bytes)
               : "memory");
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
          "r"(smem_addr(dst)),
      "l"(src), "r"(bytes), "r"(smem_addr(bar))
      : "memory");
}

__device__ __forceinline__ uint64_t global_ns() {
  uint64_t t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Waits for the barrier phase with parity `parity` to complete; gives up after about one
// second (each poll may suspend the thread for at most 1 us, and the poll count and the
// global timer are both bounded) and returns false (the caller reports it and carries on).
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity) {
  const uint32_t a = smem_addr(bar);
  const uint64_t t0 = global_ns();
  for (int it = 0; it < (1 << 20); ++it) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n"
        " selp.u32 %0, 1, 0, p;\n}" : "=r"(done) : "r"(a), "r"(parity), "r"(1000u) : "memory");
    if (done) return true;
    if ((it & 63) == 63 && global_ns() - t0 > 1000000000ull) return false;
  }
  return false;
}

}  // namespace dvm
