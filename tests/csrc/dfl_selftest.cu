// Self-test of the FP32-pipe FP64-accurate arithmetic (2d_dvm_microflows_gb300/csrc/
// dfloat.cuh) against FP64 on the device: prints the largest relative errors.
#include <cmath>
#include <cstdio>
#include <cstdint>
#include <vector>

#include "dfloat.cuh"

using namespace dvm;

__global__ void k_check(const double* x, const double* y, int n, double* err) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= n) return;
  const double a = x[t], b = y[t];
  const dfl da = dfl_from_double(a), db = dfl_from_double(b);
  const double e0 = fabs(dfl_to_double(da) - a) / fabs(a);
  const double e1 = fabs(dfl_to_double(dfl_add(da, db)) - (a + b)) / (fabs(a) + fabs(b));
  const double e2 = fabs(dfl_to_double(dfl_mul(da, db)) - a * b) / fabs(a * b);
  dacc s;
  dacc_zero(s);
  dacc_fma(s, da, db);
  dacc_add(s, db);
  const double e3 = fabs(dacc_to_double(s) - (a * b + b)) / (fabs(a * b) + fabs(b));
  err[4 * t + 0] = e0;
  err[4 * t + 1] = e1;
  err[4 * t + 2] = e2;
  err[4 * t + 3] = e3;
}

// One thread sums n positive values in a dacc; the host compares with a long-double sum.
__global__ void k_sum(const double* x, int n, double* out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  dacc s;
  dacc_zero(s);
  for (int i = 0; i < n; ++i) dacc_add(s, dfl_from_double(x[i]));
  out[0] = dacc_to_double(s);
}

int main() {
  const int n = 1 << 16;
  std::vector<double> x(n), y(n);
  uint64_t st = 88172645463325252ull;
  auto rnd = [&]() {
    st ^= st << 13; st ^= st >> 7; st ^= st << 17;
    return static_cast<double>(st >> 11) * (1.0 / 9007199254740992.0);
  };
  for (int i = 0; i < n; ++i) {
    // magnitudes 1e-25 .. 1e3, both signs (products stay above 2^-100, where the lo part
    // of a pair is still a normal float)
    x[i] = (rnd() < 0.5 ? -1.0 : 1.0) * std::pow(10.0, -25.0 + 28.0 * rnd()) * (1.0 + rnd());
    y[i] = (rnd() < 0.5 ? -1.0 : 1.0) * std::pow(10.0, -3.0 + 6.0 * rnd()) * (1.0 + rnd());
  }
  double *dx, *dy, *de;
  cudaMalloc(&dx, n * sizeof(double));
  cudaMalloc(&dy, n * sizeof(double));
  cudaMalloc(&de, 4 * n * sizeof(double));
  cudaMemcpy(dx, x.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  cudaMemcpy(dy, y.data(), n * sizeof(double), cudaMemcpyHostToDevice);
  k_check<<<(n + 255) / 256, 256>>>(dx, dy, n, de);
  std::vector<double> e(4 * n);
  cudaMemcpy(e.data(), de, 4 * n * sizeof(double), cudaMemcpyDeviceToHost);
  double mx[4] = {0, 0, 0, 0};
  for (int i = 0; i < n; ++i)
    for (int q = 0; q < 4; ++q) mx[q] = std::fmax(mx[q], e[4 * i + q]);
  // a positive sum of 256 values spanning 1e-20 .. 1
  const int m = 256;
  std::vector<double> p(m);
  long double ref = 0.0L;
  for (int i = 0; i < m; ++i) {
    p[i] = std::pow(10.0, -20.0 + 20.0 * rnd());
    ref += p[i];
  }
  cudaMemcpy(dx, p.data(), m * sizeof(double), cudaMemcpyHostToDevice);
  k_sum<<<1, 32>>>(dx, m, de);
  double got = 0.0;
  cudaMemcpy(&got, de, sizeof(double), cudaMemcpyDeviceToHost);
  const double esum = std::fabs(got - static_cast<double>(ref)) / static_cast<double>(ref);
  const cudaError_t ce = cudaDeviceSynchronize();
  std::printf("%s %.3e %.3e %.3e %.3e %.3e\n", ce == cudaSuccess ? "ok" : "fail", mx[0], mx[1],
              mx[2], mx[3], esum);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(de);
  return ce == cudaSuccess ? 0 : 1;
}
