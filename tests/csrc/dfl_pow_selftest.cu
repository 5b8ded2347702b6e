// Self-test of the pair power function dfl_pow (2d_dvm_microflows_gb300/csrc/dfloat.cuh)
// against the FP64 pow on the device: x^q for x over the range of squared relative speeds
// and the exponents (2 - 2 omega)/2 of the molecular models; prints the largest relative
// error.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <vector>

#include "dfloat.cuh"

using namespace dvm;

__global__ void k_pow(const double* x, int n, double q, double* err) {
  __shared__ float2 tab[kExp2TabN];
  for (int t = threadIdx.x; t < kExp2TabN; t += blockDim.x) tab[t] = exp2_table_entry(t);
  __syncthreads();
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const dfl xd = dfl_from_double(x[t]);
  const double got = dfl_to_double(dfl_pow(dfl_norm(xd.hi, xd.lo), flt3_from_double(q), tab));
  const double want = pow(x[t], q);
  err[t] = fabs(got - want) / want;
}

int main() {
  const int n = 1 << 18;
  std::vector<double> x(n);
  uint64_t st = 0x9E3779B97F4A7C15ull;
  auto rnd = [&]() {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return static_cast<double>(st >> 11) * (1.0 / 9007199254740992.0);
  };
  // |g|^2 from 1e-20 to 1e5 (log-uniform), and values near 1 and near powers of two
  for (int i = 0; i < n; ++i) {
    if (i % 4 == 0) x[i] = 1.0 + (rnd() - 0.5) * 1e-3;
    else if (i % 4 == 1) x[i] = std::ldexp(1.0 + (rnd() - 0.5) * 1e-6, static_cast<int>(rnd() * 30) - 15);
    else x[i] = std::pow(10.0, -20.0 + 25.0 * rnd());
  }
  double *dx, *de;
  cudaMalloc(&dx, n * sizeof(double));
  cudaMalloc(&de, n * sizeof(double));
  cudaMemcpy(dx, x.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  // (2 - 2 omega)/2 for VHS omega 0.81, 0.74, 0.75, 0.95, 0.55, and 1/alpha for VSS alpha
  // 1.4 and 1.01
  const double qs[] = {0.5 * (2.0 - 2.0 * 0.81), 0.5 * (2.0 - 2.0 * 0.74), 0.25, 0.5 * 0.1,
                       0.45, 1.0 / 1.4, 1.0 / 1.01};
  bool ok = true;
  std::printf("ok");
  for (double q : qs) {
    k_pow<<<(n + 255) / 256, 256>>>(dx, n, q, de);
    std::vector<double> e(n);
    if (cudaMemcpy(e.data(), de, n * sizeof(double), cudaMemcpyDeviceToHost) != cudaSuccess) ok = false;
    double mx = 0.0;
    for (int i = 0; i < n; ++i) mx = std::fmax(mx, e[i]);
    std::printf(" %.3e", mx);
  }
  std::printf("\n");
  return ok ? 0 : 1;
}
