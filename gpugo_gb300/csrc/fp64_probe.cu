// fp64_probe.cu -- standalone measurement of the FP64 execution model that the
// kernels are designed around: cycles per FP64 warp instruction for dependent and
// independent chains, with 1, 8 or 32 active lanes and 1-16 warps in one block,
// and the cost of the interval primitives of ia.cuh for one warp.
//
// Build and run (one GPU):
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 --fmad=false -std=c++17 \
//        -o fp64_probe gpugo_gb300/csrc/fp64_probe.cu && ./fp64_probe
#include <cstdio>
#include <cuda_runtime.h>

#include "ia.cuh"

using namespace gg;

__global__ void dep_chain(double* out, long long* cyc, int n, int active, double seed) {
  const int lane = threadIdx.x & 31;
  double x = seed + threadIdx.x, y = 1e-9;
  const long long t0 = clock64();
  if (lane < active)
    for (int i = 0; i < n; ++i) x = __dadd_rn(x, y);
  __syncwarp();
  const long long t1 = clock64();
  out[blockIdx.x * blockDim.x + threadIdx.x] = x;
  if (lane == 0) cyc[threadIdx.x / 32] = t1 - t0;
}

__global__ void indep8(double* out, long long* cyc, int n, int active, double seed) {
  const int lane = threadIdx.x & 31;
  double x0 = seed + threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3;
  double x4 = x0 + 4, x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  const double y = 1e-9;
  const long long t0 = clock64();
  if (lane < active)
    for (int i = 0; i < n / 8; ++i) {
      x0 = __dadd_rn(x0, y); x1 = __dadd_rn(x1, y); x2 = __dadd_rn(x2, y); x3 = __dadd_rn(x3, y);
      x4 = __dadd_rn(x4, y); x5 = __dadd_rn(x5, y); x6 = __dadd_rn(x6, y); x7 = __dadd_rn(x7, y);
    }
  __syncwarp();
  const long long t1 = clock64();
  out[blockIdx.x * blockDim.x + threadIdx.x] = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (lane == 0) cyc[threadIdx.x / 32] = t1 - t0;
}

// one warp, a dependent chain of calls of an interval primitive
#define PRIM(name, decl, step, res)                                       \
  __global__ void name(double* out, long long* cyc, int n, double seed) { \
    decl;                                                                 \
    const long long t0 = clock64();                                       \
    for (int i = 0; i < n; ++i) { step; }                                 \
    const long long t1 = clock64();                                       \
    out[threadIdx.x] = res;                                               \
    if (threadIdx.x == 0) cyc[0] = t1 - t0;                               \
  }
PRIM(p_dadd_ru, double x = seed, x = __dadd_ru(x, 1e-9), x)
PRIM(p_dmul_rd, double x = seed, x = __dmul_rd(x, 1.0000001), x)
PRIM(p_dsqrt, double x = seed + 2.0, x = __dadd_rn(__dsqrt_rn(x), 1.5), x)
PRIM(p_drcp, double x = seed + 2.0, x = __dadd_rn(__drcp_rd(x), 1.5), x)
PRIM(p_cvt, double x = seed, x = (double)__double2float_rn(x) + 0.5, x)
PRIM(p_mul_signs, iv a = mk(seed, seed * 1.5); iv b = mk(0.999, 1.001), a = mul(a, b), a.lo + a.hi)
PRIM(p_mul_straddle, iv a = mk(-seed, seed * 1.5); iv b = mk(-0.999, 1.001), a = mul(a, b), a.lo + a.hi)
PRIM(p_mul4, iv a = mk(-seed, seed * 1.5); iv b = mk(-0.999, 1.001), a = mul4(a, b), a.lo + a.hi)
PRIM(p_exp, double x = seed * 1e-3, x = gg_exp(x) * 1e-3, x)
PRIM(p_cos_iv, iv a = mk(seed, seed + 0.1), iv c = cos_iv(a); a = mk(c.lo + 0.5, c.hi + 0.6), a.lo + a.hi)

typedef void (*ChainK)(double*, long long*, int, int, double);
typedef void (*PrimK)(double*, long long*, int, double);

int main() {
  double* out;
  long long* cyc;
  if (cudaMalloc(&out, 8 << 20) != cudaSuccess || cudaMalloc(&cyc, 8 << 10) != cudaSuccess) return 1;
  const int n = 4096;
  struct { const char* name; ChainK k; } chains[] = {{"dadd dependent", dep_chain}, {"dadd 8 independent", indep8}};
  const int lanes[] = {1, 8, 32}, warps[] = {1, 4, 8, 16};
  for (auto& c : chains)
    for (int w : warps)
      for (int a : lanes) {
        c.k<<<1, 32 * w>>>(out, cyc, n, a, 1.0);
        c.k<<<1, 32 * w>>>(out, cyc, n, a, 1.0);
        if (cudaDeviceSynchronize() != cudaSuccess) return 1;
        long long h[16];
        cudaMemcpy(h, cyc, 8 * w, cudaMemcpyDeviceToHost);
        long long mx = 0;
        for (int i = 0; i < w; ++i) mx = h[i] > mx ? h[i] : mx;
        printf("%-20s warps %2d lanes %2d : %6.1f cycles per op per warp\n", c.name, w, a, (double)mx / n);
      }
  struct { const char* name; PrimK k; } prims[] = {
      {"dadd.ru", p_dadd_ru}, {"dmul.rd", p_dmul_rd}, {"dsqrt.rn (+dadd)", p_dsqrt}, {"drcp.rd (+dadd)", p_drcp},
      {"f64->f32->f64 (+dadd)", p_cvt}, {"mul, signs known", p_mul_signs}, {"mul, one straddles", p_mul_straddle},
      {"mul4", p_mul4}, {"gg_exp", p_exp}, {"cos_iv", p_cos_iv}};
  const int m = 512;
  for (auto& q : prims) {
    q.k<<<1, 32>>>(out, cyc, m, 1.25);
    q.k<<<1, 32>>>(out, cyc, m, 1.25);
    if (cudaDeviceSynchronize() != cudaSuccess) return 1;
    long long c;
    cudaMemcpy(&c, cyc, 8, cudaMemcpyDeviceToHost);
    printf("%-22s %8.1f cycles per call (%5.1f FP64-instruction slots of 64 cycles)\n", q.name, (double)c / m,
           (double)c / m / 64.0);
  }
  cudaError_t e = cudaGetLastError();
  printf("status %s\n", cudaGetErrorString(e));
  return e != cudaSuccess;
}
