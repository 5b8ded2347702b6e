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
#include <cuda_runtime.h>

#include "dvm_internal.h"

namespace dvm {

// ----------------------------------------------------------------------------------------
// k_cdf: one CTA per cell.
// VR: collisions/variance_reduction.f90:234-496. FMC: collisions/full_mc.f90:110-180.
constexpr int kCdfThreads = 1024;

__device__ long long num_coll_pairs(const CollParams& cp, double beta3_min, double densA,
                                    double densB, double temp) {
  // compute_num_coll_pairs, collisions/collision_utilities.f90:106-140 (n = m)
  const double rms_sq = cp.coln_rms * cp.coln_rms;
  const double b3a = beta3_min * pow(cp.mass, 3.0 / 2.0);
  const double b3 = 0.5 * (b3a + b3a);
  double ct = 0.5 * (temp + temp);
  ct = pow(ct, 2.0 / 3.0);
  const double val = (0.5 * cp.dt * ct * densA * densB) / (cp.Kn * rms_sq * b3);
  if (!(val < 9.0e18)) return 0;
  return llround(val);
}

__global__ void __launch_bounds__(kCdfThreads) k_cdf(CdfArgs a) {
  __shared__ double s_scan[64];
  __shared__ double s_par[6];
  __shared__ int s_new;
  __shared__ int s_right[2][kNRef];
  const GridInfo& g = a.g;
  const int cell = blockIdx.x;
  const int nv = g.nv;
  const size_t cs = static_cast<size_t>(cell) * (nv + 1);
  const double* f = a.f + static_cast<size_t>(cell) * nv;
  const double* P = a.props + static_cast<size_t>(cell) * DVM_NPROP;
  double* eq = a.eq_pre + cs;
  double* ce = a.cum_eq + cs;
  double* cd = a.cum_dev + cs;
  double* kin = a.kin + cs;
  const bool vr = (a.cp.method == DVM_COLL_VR);
  const int NX = g.nx, NXY = g.nx * g.ny;

  if (vr) {
    if (threadIdx.x == 0) {
      const double dens = P[DVM_P_DENS], u = P[DVM_P_U], v = P[DVM_P_V], w = P[DVM_P_W];
      double temp = P[DVM_P_SPECIES_TEMP];
      if (temp < kDoubleTol) temp = P[DVM_P_TEMP];
      const double mc = (dens > 0.0) ? dens * maxwell_coeff(a.cp.mass, temp, a.cp.pi) : 0.0;
      double* cache = a.eq_cache + static_cast<size_t>(cell) * 4;
      const double tol = a.cp.cdf_tolerance;
      // new_eq_flag, variance_reduction.f90:316-322 (w is neither tested nor stored)
      const int nw = (fabs(dens - cache[0]) > tol * dens || fabs(u - cache[1]) > tol * u ||
                      fabs(v - cache[2]) > tol * v || fabs(temp - cache[3]) > tol * temp);
      if (nw) { cache[0] = dens; cache[1] = u; cache[2] = v; cache[3] = temp; }
      s_new = nw;
      s_par[0] = mc; s_par[1] = u; s_par[2] = v; s_par[3] = w; s_par[4] = temp;
    }
    __syncthreads();
    if (s_new) {
      const double mc = s_par[0], u = s_par[1], v = s_par[2], w = s_par[3], temp = s_par[4];
      double carry = 0.0;
      if (threadIdx.x == 0) eq[0] = 0.0;
      for (int base = 0; base < nv; base += kCdfThreads) {
        const int l = base + threadIdx.x;
        double pe = 0.0, dummy = 0.0, te, td;
        if (l < nv) {
          const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
          const double b3 = g.bx[i] * g.by[j] * g.bz[k];
          pe = (temp > 0.0) ? maxwellian(g.x[i], g.y[j], g.z[k], mc, a.cp.mass, u, v, w, temp)
                            : 0.0;
          pe = pe * b3;
        }
        block_scan2(pe, dummy, te, td, s_scan);
        if (l < nv) eq[l + 1] = carry + pe;
        carry += te;
      }
      __syncthreads();
    }
    double carry_e = 0.0, carry_d = 0.0;
    for (int base = 0; base < nv; base += kCdfThreads) {
      const int l = base + threadIdx.x;
      double pe = 0.0, pn = 0.0;
      if (l < nv) {
        pe = eq[l + 1] - eq[l];
        pn = f[l] - pe;
        kin[l + 1] = pn;
      }
      double ad = fabs(pn), te, td;
      block_scan2(pe, ad, te, td, s_scan);
      if (l < nv) { ce[l + 1] = carry_e + pe; cd[l + 1] = carry_d + ad; }
      carry_e += te;
      carry_d += td;
    }
  } else {
    double carry = 0.0;
    for (int base = 0; base < nv; base += kCdfThreads) {
      const int l = base + threadIdx.x;
      double v = 0.0, dummy = 0.0, t0, t1;
      if (l < nv) { v = f[l]; kin[l + 1] = v; }
      double av = fabs(v);
      block_scan2(av, dummy, t0, t1, s_scan);
      if (l < nv) cd[l + 1] = carry + av;
      carry += t0;
    }
  }
  if (threadIdx.x == 0) { ce[0] = 0.0; cd[0] = 0.0; kin[0] = 0.0; }
  __syncthreads();

  // Bucket tables, variance_reduction.f90:471-493: right(r) is the first l >= 1 with
  // cum(l) >= r*max (the reference's running pointer reaches the same l because both the
  // CDF and the targets are nondecreasing); left(r) = right(r-1) - 1; right(1000) = n.
  const int ntab = vr ? 2 : 1;
  for (int t = 0; t < ntab; ++t) {
    const double* cum = (vr && t == 0) ? ce : cd;
    const double mx = 0.001 * cum[nv];
    for (int r = threadIdx.x + 1; r <= kNRef; r += kCdfThreads) {
      const double target = static_cast<double>(r) * mx;
      int lo = 1, hi = nv + 1;
      while (lo < hi) {
        const int mid = lo + (hi - lo) / 2;
        if (target > cum[mid]) lo = mid + 1; else hi = mid;
      }
      s_right[t][r - 1] = lo;
    }
  }
  __syncthreads();
  for (int t = 0; t < ntab; ++t) {
    int2* ref = ((vr && t == 0) ? a.ref_eq : a.ref_dev) + static_cast<size_t>(cell) * kNRef;
    for (int r = threadIdx.x + 1; r <= kNRef; r += kCdfThreads) {
      int2 e;
      e.x = (r == 1) ? 0 : s_right[t][r - 2] - 1;
      e.y = (r == kNRef) ? nv : s_right[t][r - 1];
      ref[r - 1] = e;
    }
  }

  // Sample plan of this cell-step.
  if (threadIdx.x == 0) {
    CellPlan pl;
    const CollParams& cp = a.cp;
    if (vr) {
      const double dens = P[DVM_P_DENS], temp = P[DVM_P_SPECIES_TEMP];
      const double eq_dens = ce[nv], neq_dens = cd[nv];
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
        for (int q = 0; q < 3; ++q)
          pl.num[q] = (dens > 0.0) ? num_coll_pairs(cp, g.beta3_min, dA[q], dB[q], temp) : 0;
      }
      for (int q = 0; q < 3; ++q)
        pl.factor[q] = (pl.num[q] > 0)
                           ? fc * cp.sigma * nA[q] * nB[q] / static_cast<double>(pl.num[q])
                           : 0.0;
    } else {
      const double dens = P[DVM_P_DENS], temp = P[DVM_P_TEMP];
      const double neg = 0.5 * (dens - cd[nv]);
      const double absd = dens - 2.0 * neg;
      long long num;
      if (a.pairs.active) num = a.pairs.count[0];
      else if (cp.samples_mode == DVM_SAMPLES_FIXED) num = (dens > 0.0) ? cp.samples_per_step : 0;
      else num = (dens > 0.0) ? num_coll_pairs(cp, g.beta3_min, absd / dens, absd / dens, temp) : 0;
      double factor = (num > 0) ? (cp.dt / cp.Kn) * cp.sigma * absd * absd / static_cast<double>(num)
                                : 0.0;
      factor = 0.5 * factor;
      pl.num[0] = num; pl.num[1] = 0; pl.num[2] = 0;
      pl.factor[0] = factor; pl.factor[1] = 0.0; pl.factor[2] = 0.0;
    }
    a.plan[cell] = pl;
  }
}

cudaError_t launch_cdf(const CdfArgs& a, cudaStream_t s) {
  k_cdf<<<a.ncells, kCdfThreads, 0, s>>>(a);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// k_plan: chunk offsets of every (cell, sub-integral) for the persistent collide kernel.
__global__ void __launch_bounds__(1024) k_plan(int ncells, const CellPlan* plan,
                                               long long* chunk_off, long long* total_samples) {
  __shared__ long long s_w[32];
  __shared__ long long s_carry, s_samples;
  const int n = 3 * ncells;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (threadIdx.x == 0) { s_carry = 0; s_samples = 0; }
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int e = base + threadIdx.x;
    long long num = 0;
    if (e < n) num = plan[e / 3].num[e % 3];
    long long ch = (num + kCollideChunk - 1) / kCollideChunk;
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
    if (num > 0) atomicAdd(reinterpret_cast<unsigned long long*>(&s_samples),
                           static_cast<unsigned long long>(num));
    __syncthreads();
    if (threadIdx.x == 0) s_carry += s_w[31];
    __syncthreads();
  }
  if (threadIdx.x == 0) { chunk_off[n] = s_carry; *total_samples = s_samples; }
}

cudaError_t launch_plan(int ncells, const CellPlan* plan, long long* chunk_off,
                        long long* total_samples, cudaStream_t s) {
  k_plan<<<1, 1024, 0, s>>>(ncells, plan, chunk_off, total_samples);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// k_collide: persistent; a chunk is kCollideChunk consecutive samples of one
// (cell, sub-integral). One thread per sample.
//
// GB300 runs FP64 at 1/64 of its FP32 rate and this kernel is bound by that pipe, so it
// keeps the reference's arithmetic where it decides a result and moves the rest off the
// FP64 pipe: order-preserving integer keys for every search compare, tables of node
// differences / reciprocals / remap denominator terms, a table of g and g^(2-2 omega)
// on cubic uniform grids, and the exact 1/2 mass ratios of like-species pairs. Each of
// these changes a value by at most a few ulps; the parity bar (1e-12 of max|f| against
// the restatement) checks the sum.
__device__ __forceinline__ void scatter(double* f, const Stencil& s, double w) {
#pragma unroll
  for (int q = 0; q < 7; ++q)
    if (s.node[q] >= 0) atomicAdd(f + s.node[q], w * s.mass[q]);
}

// Integer key with the order of the doubles (-0.0 folded onto +0.0).
__device__ __forceinline__ long long okey(double d) {
  long long b = __double_as_longlong(d);
  if (b == static_cast<long long>(0x8000000000000000ULL)) b = 0;
  return b >= 0 ? b : (b ^ 0x7FFFFFFFFFFFFFFFLL);
}

// referenced_search with integer compares (the CDF and the target are nonnegative).
__device__ __forceinline__ int referenced_search_keys(const double* __restrict__ cum,
                                                      const int2* __restrict__ ref, int n,
                                                      double R, uint32_t& bad) {
  if (R < kDoubleTol) return 0;
  int i = static_cast<int>(ceil(R * 1000.0));
  i = i < 1 ? 1 : (i > kNRef ? kNRef : i);
  const int2 lr = __ldg(ref + i - 1);
  int left = lr.x, right = lr.y;
  int idx = left + (right - left) / 2;
  if (left == right) return idx < n ? idx : n - 1;
  const long long* ck = reinterpret_cast<const long long*>(cum);
  const long long adj = okey(R * __ldg(cum + n));
  for (int it = 0; it < kMaxSearchIters; ++it) {
    if (idx < 0 || idx >= n) break;
    const long long c0 = okey(__longlong_as_double(__ldg(ck + idx)));
    if (adj > c0 && adj <= okey(__longlong_as_double(__ldg(ck + idx + 1)))) return idx;
    if (adj > c0) left = idx; else right = idx;
    idx = left + (right - left) / 2;
  }
  bad |= DVM_EW_SEARCH;
  int lo = 0, hi = n;
  while (hi - lo > 1) {
    const int mid = lo + (hi - lo) / 2;
    if (adj > okey(__ldg(cum + mid))) lo = mid; else hi = mid;
  }
  return lo;
}

struct SmemAxes {
  const double* v[3];
  const long long* mid[3];   // keys of the midpoints between consecutive nodes
  const AxisEntry* tab[3];
  int n[3];
};

// One axis of compute_remapping_quantities: nearest node (:146-183). The reference's
// binary_search_with_first_guess returns the node nearest to u, the lower one on a tie,
// and the first or last node outside the grid; here the guess nint(factor*(u - v_min)) is
// walked to that node with integer compares against the keys of the midpoints between
// nodes (mid[i] = (v[i] + v[i+1])/2). The choice can differ from the reference's only for
// u within an ulp of a midpoint.
__device__ __forceinline__ int nearest(const SmemAxes& A, int ax, double u, double vmin,
                                       double factor, int& corner, int& bad) {
  const int mx = A.n[ax] - 1;
  const long long* mid = A.mid[ax];
  const long long vk = okey(u);
  // the guess only starts the walk, so FP32 is enough for it
  int o = __float2int_rn(static_cast<float>(factor) *
                         (static_cast<float>(u) - static_cast<float>(vmin)));
  o = o < 0 ? 0 : (o > mx ? mx : o);
  if (u != u) bad |= 1;  // NaN velocity: the reference's search would not return
  int it = 0;
  while (o > 0 && vk <= mid[o - 1] && it++ < kMaxAxis) --o;
  while (o < mx && vk > mid[o] && it++ < kMaxAxis) ++o;
  if (o >= mx) { o = mx; corner++; }
  else if (o <= 0) { o = 0; corner++; }
  return o;
}

// Reciprocal from an FP32 seed and two Newton steps (within an ulp or two of 1/d).
__device__ __forceinline__ double fast_rcp(double d) {
  const double ad = fabs(d);
  if (!(ad > 1e-30 && ad < 1e30)) return 1.0 / d;
  double r = static_cast<double>(__frcp_rn(static_cast<float>(d)));
  double e = fma(-d, r, 1.0);
  r = fma(r, e, r);
  e = fma(-d, r, 1.0);
  return fma(r, e, r);
}

// compute_remapping_quantities (collisions/remapping.f90:92-394) with tabulated
// differences, reciprocals and denominator terms.
__device__ __forceinline__ int remap_fast(const GridInfo& g, const SmemAxes& A, double u,
                                          double v, double w, double f_off, Stencil& s) {
  int corner = 0, bad = 0;
  int o_i = nearest(A, 0, u, g.xv_min, g.xv_factor, corner, bad);
  int o_j = nearest(A, 1, v, g.yv_min, g.yv_factor, corner, bad);
  int o_k = nearest(A, 2, w, g.zv_min, g.zv_factor, corner, bad);
  const int i_max = g.nx - 1, j_max = g.ny - 1, k_max = g.nz - 1;
  if (corner == 3) {
    o_i -= isign1(o_i - 1);
    o_j -= isign1(o_j - 1);
    o_k -= isign1(o_k - 1);
  }
  const double* x = A.v[0];
  const double* y = A.v[1];
  const double* z = A.v[2];
  const double ox = x[o_i], oy = y[o_j], oz = z[o_k];
  const double a = u - ox, b = v - oy, c = w - oz;
  int sa = isgn(a), sb = isgn(b), sc = isgn(c);
  if (o_i + sa > i_max || o_i + sa < 0) {
    sa = -1 * sa;
    find_boundary_stencil(sa, sb, sc, a, o_i, o_j, o_k, x, y, z, 0, i_max, 0, j_max, 0, k_max);
  }
  if (o_j + sb > j_max || o_j + sb < 0) {
    sb = -1 * sb;
    find_boundary_stencil(sb, sa, sc, b, o_j, o_i, o_k, y, x, z, 0, j_max, 0, i_max, 0, k_max);
  }
  if (o_k + sc > k_max || o_k + sc < 0) {
    sc = -1 * sc;
    find_boundary_stencil(sc, sb, sa, c, o_k, o_j, o_i, z, y, x, 0, k_max, 0, j_max, 0, i_max);
  }
  const int fx = (o_i - sa <= i_max && o_i - sa >= 0);
  const int fy = (o_j - sb <= j_max && o_j - sb >= 0);
  const int fz = (o_k - sc <= k_max && o_k - sc >= 0);
  // per-axis differences, reciprocal of the interior difference, denominator term
  double int_x, inv_x, ext_x = 0.0, t_x = 0.0;
  if (sa >= -kTabS && sa <= kTabS) {
    const AxisEntry& e = A.tab[0][o_i];
    int_x = e.D[kTabS + sa]; inv_x = e.invD[kTabS + sa];
    if (fx) { ext_x = e.D[kTabS - sa]; t_x = e.T[kTabS + sa]; }
  } else {
    int_x = x[o_i + sa] - ox; inv_x = 1.0 / int_x;
    if (fx) { ext_x = x[o_i - sa] - ox; t_x = ext_x * (ext_x - int_x); }
  }
  double int_y, inv_y, ext_y = 0.0, t_y = 0.0;
  if (sb >= -kTabS && sb <= kTabS) {
    const AxisEntry& e = A.tab[1][o_j];
    int_y = e.D[kTabS + sb]; inv_y = e.invD[kTabS + sb];
    if (fy) { ext_y = e.D[kTabS - sb]; t_y = e.T[kTabS + sb]; }
  } else {
    int_y = y[o_j + sb] - oy; inv_y = 1.0 / int_y;
    if (fy) { ext_y = y[o_j - sb] - oy; t_y = ext_y * (ext_y - int_y); }
  }
  double int_z, inv_z, ext_z = 0.0, t_z = 0.0;
  if (sc >= -kTabS && sc <= kTabS) {
    const AxisEntry& e = A.tab[2][o_k];
    int_z = e.D[kTabS + sc]; inv_z = e.invD[kTabS + sc];
    if (fz) { ext_z = e.D[kTabS - sc]; t_z = e.T[kTabS + sc]; }
  } else {
    int_z = z[o_k + sc] - oz; inv_z = 1.0 / int_z;
    if (fz) { ext_z = z[o_k - sc] - oz; t_z = ext_z * (ext_z - int_z); }
  }
  const int flag = fx + 2 * fy + 4 * fz;
  double den = 0.0;
  if (fx) den = t_x;
  if (fy) den = den + t_y;
  if (fz) den = den + t_z;
  double f_e = 0.0;
  if (flag == 0) bad |= 2;
  else f_e = f_off * (a * a + b * b + c * c - a * int_x - b * int_y - c * int_z) * fast_rcp(den);
  const double f_ex = fx ? f_e : 0.0, f_ey = fy ? f_e : 0.0, f_ez = fz ? f_e : 0.0;
  const double f_ix = (f_off * a - f_ex * ext_x) * inv_x;
  const double f_iy = (f_off * b - f_ey * ext_y) * inv_y;
  const double f_iz = (f_off * c - f_ez * ext_z) * inv_z;
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

struct CollideSmem {
  size_t axes, keys, tabs, gtab, trig, total;
};

__host__ __device__ inline CollideSmem collide_smem_layout(const GridInfo& g, const CollTables& t) {
  CollideSmem L;
  const size_t nsum = static_cast<size_t>(g.nx + g.ny + g.nz);
  L.axes = 0;
  L.keys = L.axes + nsum * sizeof(double);
  L.tabs = L.keys + nsum * sizeof(long long);
  L.gtab = L.tabs + 3 * static_cast<size_t>(t.nmax) * sizeof(AxisEntry);
  L.gtab = (L.gtab + 15) & ~static_cast<size_t>(15);  // double2 needs 16-byte alignment
  L.trig = L.gtab + (t.gtab_smem ? static_cast<size_t>(t.gtab_n) * sizeof(double2) : 0);
  L.total = L.trig + static_cast<size_t>(kTrigN) * sizeof(double2);
  return L;
}

__global__ void __launch_bounds__(kCollideChunk) k_collide(CollideArgs a) {
  extern __shared__ __align__(16) unsigned char s_raw[];
  const GridInfo& g = a.g;
  const CollideSmem L = collide_smem_layout(g, a.t);
  double* sv = reinterpret_cast<double*>(s_raw + L.axes);
  long long* sk = reinterpret_cast<long long*>(s_raw + L.keys);
  AxisEntry* st = reinterpret_cast<AxisEntry*>(s_raw + L.tabs);
  double2* sg = reinterpret_cast<double2*>(s_raw + L.gtab);
  const int nsum = g.nx + g.ny + g.nz;
  for (int t = threadIdx.x; t < nsum; t += blockDim.x) {
    const double* ax = t < g.nx ? g.x : (t < g.nx + g.ny ? g.y : g.z);
    const int n = t < g.nx ? g.nx : (t < g.nx + g.ny ? g.ny : g.nz);
    const int i = t < g.nx ? t : (t < g.nx + g.ny ? t - g.nx : t - g.nx - g.ny);
    sv[t] = ax[i];
    sk[t] = (i + 1 < n) ? okey(0.5 * (ax[i] + ax[i + 1])) : 0x7FFFFFFFFFFFFFFFLL;
  }
  {
    const double* src = reinterpret_cast<const double*>(a.t.axis);
    double* dst = reinterpret_cast<double*>(st);
    const int n = 3 * a.t.nmax * static_cast<int>(sizeof(AxisEntry) / sizeof(double));
    for (int t = threadIdx.x; t < n; t += blockDim.x) dst[t] = src[t];
  }
  if (a.t.gtab_smem)
    for (int t = threadIdx.x; t < a.t.gtab_n; t += blockDim.x) sg[t] = a.t.gtab[t];
  double2* strig = reinterpret_cast<double2*>(s_raw + L.trig);
  for (int t = threadIdx.x; t < kTrigN; t += blockDim.x) strig[t] = a.t.trig[t];
  __syncthreads();
  SmemAxes A;
  A.v[0] = sv; A.v[1] = sv + g.nx; A.v[2] = sv + g.nx + g.ny;
  A.mid[0] = sk; A.mid[1] = sk + g.nx; A.mid[2] = sk + g.nx + g.ny;
  A.tab[0] = st; A.tab[1] = st + a.t.nmax; A.tab[2] = st + 2 * a.t.nmax;
  A.n[0] = g.nx; A.n[1] = g.ny; A.n[2] = g.nz;
  const double2* gtab = a.t.gtab_smem ? sg : a.t.gtab;

  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const int nent = 3 * a.ncells;
  const long long total = a.chunk_off[nent];
  const bool vr = (a.cp.method == DVM_COLL_VR);
  const int NR = a.cp.num_repl;
  const double vhs = 2.0 - 2.0 * (0.5 * (a.cp.omega + a.cp.omega));
  const double alpha = 0.5 * (a.cp.alpha + a.cp.alpha);
  const double ralpha = 1.0 / alpha;
  const bool vss = fabs(ralpha - 1.0) > kDoubleTol;
  // like-species pair: mass fractions m/(m+m) are exactly 1/2
  constexpr double mf = 0.5;
  uint32_t bad = 0;

  for (long long chunk = blockIdx.x; chunk < total; chunk += gridDim.x) {
    int lo = 0, hi = nent;
    while (hi - lo > 1) {
      const int mid = (lo + hi) >> 1;
      if (a.chunk_off[mid] <= chunk) lo = mid; else hi = mid;
    }
    const int cell = lo / 3, q = lo - 3 * (lo / 3);
    const CellPlan& pl = a.plan[cell];
    const long long i = (chunk - a.chunk_off[lo]) * kCollideChunk + threadIdx.x;
    if (i >= pl.num[q]) continue;
    const double factor = pl.factor[q];
    const size_t cs = static_cast<size_t>(cell) * (nv + 1);
    double* f = a.f + static_cast<size_t>(cell) * nv;

    // partners: pick_collision_partner x2 (collision_utilities.f90:142-186)
    double rA = 0.0, rB = 0.0;
    const bool rec = a.pairs.active;
    if (!rec) philox_uniform2(a.cp.seed, static_cast<uint32_t>(i), cell, a.step, q, 0u, rA, rB);
    int lA, lB;
    if (rec && a.pairs.glA[q]) {
      lA = a.pairs.glA[q][i];
      lB = a.pairs.glB[q][i];
    } else {
      if (rec) { rA = a.pairs.rA[q][i]; rB = a.pairs.rB[q][i]; }
      const bool aeq = vr && q == 0, beq = vr && q == 1;
      lA = referenced_search_keys((aeq ? a.cum_eq : a.cum_dev) + cs,
                                  (aeq ? a.ref_eq : a.ref_dev) + static_cast<size_t>(cell) * kNRef,
                                  nv, rA, bad);
      lB = referenced_search_keys((beq ? a.cum_eq : a.cum_dev) + cs,
                                  (beq ? a.ref_eq : a.ref_dev) + static_cast<size_t>(cell) * kNRef,
                                  nv, rB, bad);
    }
    const int kA = lA / NXY, jA = (lA - kA * NXY) / NX, iA = lA - kA * NXY - jA * NX;
    const int kB = lB / NXY, jB = (lB - kB * NXY) / NX, iB = lB - kB * NXY - jB * NX;
    const double xA = A.v[0][iA], yA = A.v[1][jA], zA = A.v[2][kA];
    const double xB = A.v[0][iB], yB = A.v[1][jB], zB = A.v[2][kB];
    // compute_relative_velocity (collision_utilities.f90:188-218) and g^(2-2 omega)
    double gg, g_sigma;
    if (gtab) {
      const int di = iB - iA, dj = jB - jA, dk = kB - kA;
      const int s2 = di * di + dj * dj + dk * dk;
      if (s2 == 0) continue;  // g < double_tol, variance_reduction.f90:697
      const double2 e = gtab[s2];
      gg = e.x;
      g_sigma = e.y;
    } else {
      const double gx = xB - xA, gy = yB - yA, gz = zB - zA;
      gg = sqrt(gx * gx + gy * gy + gz * gz);
      if (gg < kDoubleTol) continue;
      g_sigma = (vhs == 1.0) ? gg : pow(gg, vhs);
    }
    // signs of the deviation partners (cdf_neq%sign); FMC: sign of phi_old
    const double* kc = a.kin + cs;
    const double sA = (vr && q == 0) ? 1.0 : dsgn(__ldg(kc + lA + 1));
    const double sB = (vr && q == 1) ? 1.0 : dsgn(__ldg(kc + lB + 1));
    // vr_depletion_routine elastic part (variance_reduction.f90:1157-1166)
    const double kin1 = sA * (sB * factor * g_sigma);
    const double kin2 = sB * (sA * factor * g_sigma);
    atomicAdd(f + lA, -kin1);
    atomicAdd(f + lB, -kin2);
    // replenish_collision elastic branch (replenishing_collisions.f90:206-249)
    const double kr1 = (NR == 1) ? kin1 : kin1 / static_cast<double>(NR);
    const double kr2 = (NR == 1) ? kin2 : kin2 / static_cast<double>(NR);
    const double vc0 = mf * xA + mf * xB, vc1 = mf * yA + mf * yB, vc2 = mf * zA + mf * zB;
    // g_part(1)/g = g_part(2)/g = 1/2 for equal masses (pick_random_velocity_on_sphere
    // :343-351); the VSS branch also needs the summed |xi - v_com| components.
    const double hg = 0.5 * gg;
    for (int r = 0; r < NR; ++r) {
      double rphi, rcos;
      if (rec) {
        rphi = a.pairs.rphi[q][i * NR + r];
        rcos = a.pairs.rcos[q][i * NR + r];
      } else {
        philox_uniform2(a.cp.seed, static_cast<uint32_t>(i), cell, a.step, q, 1u + r, rphi, rcos);
      }
      // pick_random_velocity_on_sphere (collision_utilities.f90:284-352); phi = 2 pi R:
      // R = k/kTrigN + t exactly, cos/sin of 2 pi k/kTrigN from the table, of
      // th = 2 pi t (< 0.0062) by Taylor series (next terms below 1e-17), then the
      // angle-addition formulas.
      double sphi, cphi;
      {
        const double rk = floor(rphi * static_cast<double>(kTrigN));
        const int k = min(max(static_cast<int>(rk), 0), kTrigN - 1);
        const double th = a.t.two_pi * (rphi - rk * (1.0 / kTrigN));
        const double t2 = th * th;
        const double st = th * (1.0 - t2 * (1.0 / 6.0) * (1.0 - t2 * (1.0 / 20.0)));
        const double ct = 1.0 - t2 * 0.5 * (1.0 - t2 * (1.0 / 12.0) * (1.0 - t2 * (1.0 / 30.0)));
        const double2 cs = strig[k];
        cphi = cs.x * ct - cs.y * st;
        sphi = cs.y * ct + cs.x * st;
      }
      double ux, uy, uz;  // r / g: unit direction of the post-collision relative velocity
      if (vss) {
        const double ur = fabs(xA - vc0) + fabs(xB - vc0);
        const double vr_ = fabs(yA - vc1) + fabs(yB - vc1);
        const double wr = fabs(zA - vc2) + fabs(zB - vc2);
        const double ct = 2.0 * pow(rcos, ralpha) - 1.0;
        const double st = sqrt(1.0 - ct * ct);
        const double den = sqrt(vr_ * vr_ + wr * wr);
        double rx, ry, rz;
        if (den > kDoubleTol * gg) {
          rx = ct * ur + st * sphi * den;
          ry = ct * vr_ + st * (gg * wr * cphi - ur * vr_ * sphi) / den;
          rz = ct * wr - st * (gg * vr_ * cphi + ur * wr * sphi) / den;
        } else {
          rx = ct * ur;
          ry = st * cphi * ur;
          rz = st * sphi * ur;
        }
        ux = 0.5 * rx; uy = 0.5 * ry; uz = 0.5 * rz;
      } else {
        const double ct = 2.0 * rcos - 1.0;
        const double st = sqrt(1.0 - ct * ct);
        ux = hg * st * cphi;
        uy = hg * st * sphi;
        uz = hg * ct;
      }
      Stencil s;
      int rb = remap_fast(g, A, vc0 + ux, vc1 + uy, vc2 + uz, 1.0, s);
      if (rb & 2) bad |= DVM_EW_REMAP; else scatter(f, s, kr1);
      if (rb & 1) bad |= DVM_EW_SEARCH;
      rb = remap_fast(g, A, vc0 - ux, vc1 - uy, vc2 - uz, 1.0, s);
      if (rb & 2) bad |= DVM_EW_REMAP; else scatter(f, s, kr2);
      if (rb & 1) bad |= DVM_EW_SEARCH;
    }
  }
  if (bad) atomicOr(a.err, bad);
}

size_t collide_smem_bytes(const GridInfo& g, const CollTables& t) {
  return collide_smem_layout(g, t).total;
}

int collide_blocks_per_sm(size_t smem) {
  int n = 0;
  if (smem > 48 * 1024)
    cudaFuncSetAttribute(k_collide, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(smem));
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_collide, kCollideChunk, smem) !=
      cudaSuccess)
    n = 1;
  return n > 0 ? n : 1;
}

cudaError_t launch_collide(const CollideArgs& a, int grid, cudaStream_t s) {
  const size_t smem = collide_smem_bytes(a.g, a.t);
  if (smem > 48 * 1024) {
    const cudaError_t e = cudaFuncSetAttribute(
        k_collide, cudaFuncAttributeMaxDynamicSharedMemorySize, static_cast<int>(smem));
    if (e != cudaSuccess) return e;
  }
  k_collide<<<grid, kCollideChunk, smem, s>>>(a);
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
  const GridInfo& g = a.g;
  const WallEntry we = wall_entry(a, blockIdx.x);
  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const double* f = a.f + (static_cast<size_t>(we.cx) + static_cast<size_t>(a.nxs) * we.cy) * nv;
  double* gh = a.ghost + static_cast<size_t>(blockIdx.x) * nv;
  const bool xwall = (we.side == DVM_WALL_LEFT || we.side == DVM_WALL_RIGHT);
  const double* W = a.wall[we.side];
  const double T = W[DVM_WP_TEMP], u = W[DVM_WP_U], v = W[DVM_WP_V], w = W[DVM_WP_W];
  const double mc = maxwell_coeff(a.mass, T, a.pi);
  double acc2[2] = {0.0, 0.0};  // flux_in, flux_out
  for (int l = threadIdx.x; l < nv; l += blockDim.x) {
    const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
    const double vn = xwall ? g.x[i] : g.y[j];
    if (wall_incoming(g, we.side, i, j)) acc2[0] += fabs(vn) * a.acc * f[l];
    double val = 0.0;
    if (a.acc > 0.0 && wall_outgoing(g, we.side, i, j)) {
      const double b3 = g.bx[i] * g.by[j] * g.bz[k];
      const double M = maxwellian(g.x[i], g.y[j], g.z[k], mc, a.mass, u, v, w, T);
      val = M * b3;
      acc2[1] += fabs(vn) * M * b3;
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
  scatter(gh, s, dens);
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

__global__ void __launch_bounds__(256) k_convect2d(Convect2DArgs a) {
  const GridInfo& g = a.g;
  const int nv = g.nv;
  const int l = blockIdx.x * blockDim.x + threadIdx.x;
  if (l >= nv) return;
  const int cell = blockIdx.y;
  const int cx = cell % a.nxs, cy = cell / a.nxs;
  const int NX = g.nx, NXY = g.nx * g.ny;
  const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
  (void)k;
  const size_t off = static_cast<size_t>(cell) * nv + l;
  const double f0 = a.f[off];
  const double xv = g.x[i], yv = g.y[j];
  const double cfx = a.xf * xv, cfy = a.yf * yv;
  const bool perim = (cx == 0 || cy == 0 || cx == a.nxs - 1 || cy == a.nys - 1);
  double out;
  if (!perim) {
    const double px = (xv < 0.0) ? a.f[off + nv] : a.f[off - nv];
    const size_t row = static_cast<size_t>(a.nxs) * nv;
    const double py = (yv < 0.0) ? a.f[off + row] : a.f[off - row];
    out = f0 + fabs(cfx) * (px - f0) + fabs(cfy) * (py - f0);
  } else {
    const int ci = axis_class(i, g.i_neg, g.i_pos, g.i_zero, g.i_zero_flag);
    const int cj = axis_class(j, g.j_neg, g.j_pos, g.j_zero, g.j_zero_flag);
    if (ci == kClsNone || cj == kClsNone) {
      out = 0.0;
    } else {
      double gx = 0.0, gy = 0.0;
      if (ci == kClsNeg) {  // upwind is the right neighbour / right wall ghost
        if (cx < a.nxs - 1) gx = a.f[off + nv];
        else if (a.bc_right == DVM_BC2D_WALL) gx = a.ghost[static_cast<size_t>(a.base[1] + cy) * nv + l];
        else if (a.bc_right == DVM_BC2D_COUETTE) gx = a.f[static_cast<size_t>(a.nxs) * cy * nv + l];
      } else if (ci == kClsPos) {  // left neighbour / left wall ghost
        if (cx > 0) gx = a.f[off - nv];
        else if (a.bc_left == DVM_BC2D_WALL) gx = a.ghost[static_cast<size_t>(a.base[0] + cy) * nv + l];
        else if (a.bc_left == DVM_BC2D_COUETTE) gx = f0;
      }
      if (cj == kClsNeg) {  // top neighbour / top wall ghost
        if (cy < a.nys - 1) gy = a.f[off + static_cast<size_t>(a.nxs) * nv];
        else gy = a.ghost[static_cast<size_t>(a.base[3] + cx) * nv + l];
      } else if (cj == kClsPos) {  // bottom neighbour / bottom wall ghost
        if (cy > 0) gy = a.f[off - static_cast<size_t>(a.nxs) * nv];
        else gy = a.ghost[static_cast<size_t>(a.base[2] + cx) * nv + l];
      }
      const bool hx = (ci != kClsZero), hy = (cj != kClsZero);
      if (hx && hy) out = f0 + fabs(cfx) * (gx - f0) + fabs(cfy) * (gy - f0);
      else if (hy) out = f0 + fabs(cfy) * (gy - f0);
      else if (hx) out = f0 + fabs(cfx) * (gx - f0);
      else out = f0;
    }
  }
  a.fconv[off] = out;
}

cudaError_t launch_convect2d(const Convect2DArgs& a, int ncells, cudaStream_t s) {
  dim3 grid((a.g.nv + 255) / 256, ncells);
  k_convect2d<<<grid, 256, 0, s>>>(a);
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
  const int nx = blockIdx.y;
  const size_t off = static_cast<size_t>(nx) * nv + l;
  const double p0 = a.f[off];
  if (nx == 0 || nx == a.nxs - 1) { a.fconv[off] = p0; return; }
  const int i = l % g.nx;
  const double xv = g.x[i];
  const double cfl = a.factor * xv;
  a.fconv[off] = (xv < 0.0) ? p0 - cfl * (a.f[off + nv] - p0) : p0 - cfl * (p0 - a.f[off - nv]);
}

cudaError_t launch_convect1d(const Convect1DArgs& a, cudaStream_t s) {
  dim3 grid((a.g.nv + 255) / 256, a.nxs);
  k_convect1d<<<grid, 256, 0, s>>>(a);
  return cudaGetLastError();
}

// End conditions (grid_ref conditions/boundary_conditions.f90:319-1000); one CTA per end.
constexpr int kBc1dThreads = 1024;

__global__ void __launch_bounds__(kBc1dThreads) k_bc1d(Convect1DArgs a) {
  __shared__ double s_red[2 * 32];
  const GridInfo& g = a.g;
  const int e = blockIdx.x;  // 0 left, 1 right
  const int nx = (e == 0) ? 0 : a.nxs - 1;
  const int bc = a.bc[e];
  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const double* f = a.f + static_cast<size_t>(nx) * nv;
  double* fc = a.fconv + static_cast<size_t>(nx) * nv;
  const double* W = a.wall[e];
  if (bc == DVM_BC1D_SPECULAR) {  // apply_specular_wall :446-564
    for (int l = threadIdx.x; l < nv; l += blockDim.x) {
      const double xv = g.x[l % NX];
      const double fac = a.factor * xv;
      if (e == 0 && xv < 0.0) fc[l] = f[l] - fac * (f[l + nv] - f[l]);
      if (e == 1 && xv > 0.0) fc[l] = f[l] - fac * (f[l] - f[l - nv]);
    }
  } else if (bc == DVM_BC1D_INOUT) {  // apply_fixed_in_out_flow :783-913
    const double dens = W[DVM_WP_DENS], T = W[DVM_WP_TEMP], u = W[DVM_WP_U];
    const double mc = dens * maxwell_coeff(a.mass, T, a.pi);
    for (int l = threadIdx.x; l < nv; l += blockDim.x) {
      const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
      const double b3 = g.bx[i] * g.by[j] * g.bz[k];
      fc[l] = maxwellian(g.x[i], g.y[j], g.z[k], mc, a.mass, u, 0.0, 0.0, T) * b3;
    }
  } else if (bc == DVM_BC1D_ZEROGRAD) {  // apply_zero_gradient_flow :915-962
    const double* src = a.fconv + static_cast<size_t>(e == 0 ? 1 : a.nxs - 2) * nv;
    for (int l = threadIdx.x; l < nv; l += blockDim.x) fc[l] = src[l];
  } else if (bc == DVM_BC1D_DIFFUSE) {  // apply_diffuse_reflection :566-781
    const double T = W[DVM_WP_TEMP], u = W[DVM_WP_U], v = W[DVM_WP_V], w = W[DVM_WP_W];
    const double* f2 = a.f + static_cast<size_t>(e == 0 ? 1 : a.nxs - 2) * nv;
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
  k_bc1d<<<2, kBc1dThreads, 0, s>>>(a);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
// k_moments: one CTA per cell. Pass 1: n, n u (compute_density, compute_*_velocity,
// compute_avg_speed); pass 2: T, q, tau about u (compute_temperature, compute_heat_flux,
// compute_viscous_stress), dist_funcs/physical_props.f90:879-1087, 1459-1507, 1914-2071.
constexpr int kMomThreads = 256;

__global__ void __launch_bounds__(kMomThreads) k_moments(MomentArgs a) {
  __shared__ double s_red[10 * 32];
  const GridInfo& g = a.g;
  const int cell = blockIdx.x;
  const int nv = g.nv, NX = g.nx, NXY = g.nx * g.ny;
  const double* f = a.f + static_cast<size_t>(cell) * nv;
  double p1[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
  for (int l = threadIdx.x; l < nv; l += blockDim.x) {
    const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
    const double fv = f[l], x = g.x[i], y = g.y[j], z = g.z[k];
    p1[0] += fv;
    p1[1] += fv * x;
    p1[2] += fv * y;
    p1[3] += fv * z;
    p1[4] += fv * sqrt(x * x + y * y + z * z);
  }
  block_sum<5>(p1, s_red);
  const double dens = p1[0];
  double* P = a.props + static_cast<size_t>(cell) * DVM_NPROP;
  if (dens == 0.0) {
    for (int q = threadIdx.x; q < DVM_NPROP; q += blockDim.x) P[q] = 0.0;
    return;
  }
  const double u = p1[1] / dens, v = p1[2] / dens, w = p1[3] / dens;
  double p2[10] = {0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
  for (int l = threadIdx.x; l < nv; l += blockDim.x) {
    const int k = l / NXY, j = (l - k * NXY) / NX, i = l - k * NXY - j * NX;
    const double fv = f[l];
    const double cx = g.x[i] - u, cy = g.y[j] - v, cz = g.z[k] - w;
    const double csq = cx * cx + cy * cy + cz * cz;
    p2[0] += fv * csq;
    p2[1] += cx * csq * fv;
    p2[2] += cy * csq * fv;
    p2[3] += cz * csq * fv;
    p2[4] -= cx * cx * fv;
    p2[5] -= cy * cy * fv;
    p2[6] -= cz * cz * fv;
    p2[7] -= cx * cy * fv;
    p2[8] -= cx * cz * fv;
    p2[9] -= cy * cz * fv;
  }
  block_sum<10>(p2, s_red);
  if (threadIdx.x == 0) {
    const double m = a.mass;
    const double t = 2.0 * m * p2[0] / (3.0 * dens);
    const double p = 0.5 * dens * t;
    P[DVM_P_DENS] = dens; P[DVM_P_U] = u; P[DVM_P_V] = v; P[DVM_P_W] = w;
    P[DVM_P_TEMP] = t;
    P[DVM_P_SPECIES_TEMP] = (3.0 * t + 0.0 * 0.0 + 0.0 * 0.0) / (3.0 + 0.0 + 0.0);
    P[DVM_P_AVG_SPEED] = p1[4] / dens;
    P[DVM_P_PRESSURE] = p;
    P[DVM_P_QX] = p2[1] * (0.5 * m); P[DVM_P_QY] = p2[2] * (0.5 * m); P[DVM_P_QZ] = p2[3] * (0.5 * m);
    P[DVM_P_TXX] = p + m * p2[4]; P[DVM_P_TYY] = p + m * p2[5]; P[DVM_P_TZZ] = p + m * p2[6];
    P[DVM_P_TXY] = m * p2[7]; P[DVM_P_TXZ] = m * p2[8]; P[DVM_P_TYZ] = m * p2[9];
    for (int q = DVM_P_TYZ + 1; q < DVM_NPROP; ++q) P[q] = 0.0;
    uint32_t bad = 0;
    if (!isfinite(dens) || !isfinite(t)) bad |= DVM_EW_NONFINITE;
    if (!(dens > 0.0)) bad |= DVM_EW_NEGDENS;
    if (bad) atomicOr(a.err, bad);
  }
}

cudaError_t launch_moments(const MomentArgs& a, cudaStream_t s) {
  k_moments<<<a.ncells, kMomThreads, 0, s>>>(a);
  return cudaGetLastError();
}

// ----------------------------------------------------------------------------------------
__global__ void k_flush(double* buf, size_t n) {
  for (size_t t = blockIdx.x * static_cast<size_t>(blockDim.x) + threadIdx.x; t < n;
       t += static_cast<size_t>(gridDim.x) * blockDim.x)
    buf[t] = static_cast<double>(t);
}

cudaError_t launch_flush(double* buf, size_t n, cudaStream_t s) {
  k_flush<<<1216, 256, 0, s>>>(buf, n);
  return cudaGetLastError();
}

}  // namespace dvm
