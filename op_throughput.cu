// Throughput of single arithmetic operations on the GPU: FP32 and FP64 FMA,
// 32-bit integer multiply-add (low, high, and 32x32->64 wide), adds, shifts,
// leading-zero counts and FP64<->int64 conversions.  Each thread runs 8
// independent chains of 2048 operations; grid = 8 CTAs of 256 threads per
// SM.  It measures the rates the complex128 arithmetic choice rests on
// (native FP64 vs. 64-bit integer fixed point vs. float-float).
//
// Build and run (one GPU):
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o op_throughput op_throughput.cu && ./op_throughput
#include <cstdio>
#include <cstdint>
#include <cuda_runtime.h>

constexpr int ITER = 2048;
constexpr int CH = 8;

#define KERN(NAME, T, INIT, BODY, OUT)                                        \
  __global__ void NAME(T* out, T seed) {                                      \
    T a[CH];                                                                   \
    _Pragma("unroll") for (int c = 0; c < CH; ++c) a[c] = INIT;                \
    T b = seed + (T)threadIdx.x;                                               \
    for (int it = 0; it < ITER; ++it) {                                        \
      _Pragma("unroll") for (int c = 0; c < CH; ++c) { BODY; }                 \
    }                                                                          \
    T s = 0;                                                                   \
    _Pragma("unroll") for (int c = 0; c < CH; ++c) s += a[c];                  \
    if (s == (T)12345) out[threadIdx.x] = OUT;                                 \
  }

KERN(k_ffma, float, seed * c, asm volatile("fma.rn.f32 %0, %0, %1, %1;" : "+f"(a[c]) : "f"(b)), s)
KERN(k_dfma, double, seed * c, asm volatile("fma.rn.f64 %0, %0, %1, %1;" : "+d"(a[c]) : "d"(b)), s)
KERN(k_imad, int32_t, seed * c, asm volatile("mad.lo.s32 %0, %0, %1, %1;" : "+r"(a[c]) : "r"(b)), s)
KERN(k_imadhi, uint32_t, seed * c, asm volatile("mad.hi.u32 %0, %0, %1, %1;" : "+r"(a[c]) : "r"(b)), s)
KERN(k_add, uint32_t, seed * c, asm volatile("add.u32 %0, %0, %1;" : "+r"(a[c]) : "r"(b)), s)
KERN(k_shf, uint32_t, seed * c, asm volatile("shf.l.wrap.b32 %0, %0, %1, 7;" : "+r"(a[c]) : "r"(b)), s)
KERN(k_clz, uint32_t, seed * c, asm volatile("{.reg .u32 t; clz.b32 t, %0; add.u32 %0, %0, t;}" : "+r"(a[c])), s)
KERN(k_add64, uint64_t, seed * c, asm volatile("add.u64 %0, %0, %1;" : "+l"(a[c]) : "l"(b)), s)

// d64 = a32 * b32 + d64
__global__ void k_imadwide(int64_t* out, int32_t seed) {
  int64_t a[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) a[c] = seed * c;
  int32_t x = seed + threadIdx.x, y = seed ^ threadIdx.x;
  for (int it = 0; it < ITER; ++it) {
#pragma unroll
    for (int c = 0; c < CH; ++c) asm volatile("mad.wide.s32 %0, %1, %2, %0;" : "+l"(a[c]) : "r"(x), "r"(y));
  }
  int64_t s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += a[c];
  if (s == 12345) out[threadIdx.x] = s;
}
__global__ void k_imadwideu(uint64_t* out, uint32_t seed) {
  uint64_t a[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) a[c] = seed * c;
  uint32_t x = seed + threadIdx.x, y = seed ^ threadIdx.x;
  for (int it = 0; it < ITER; ++it) {
#pragma unroll
    for (int c = 0; c < CH; ++c) asm volatile("mad.wide.u32 %0, %1, %2, %0;" : "+l"(a[c]) : "r"(x), "r"(y));
  }
  uint64_t s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += a[c];
  if (s == 12345) out[threadIdx.x] = s;
}
// double <-> int64 conversions (round trip chain)
__global__ void k_cvt(double* out, double seed) {
  double a[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) a[c] = seed * (c + 1);
  for (int it = 0; it < ITER; ++it) {
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      int64_t t;
      asm volatile("cvt.rzi.s64.f64 %0, %1;" : "=l"(t) : "d"(a[c]));
      asm volatile("cvt.rn.f64.s64 %0, %1;" : "=d"(a[c]) : "l"(t));
    }
  }
  double s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += a[c];
  if (s == 12345) out[threadIdx.x] = s;
}
// f32 <-> s32 conversions
__global__ void k_cvt32(float* out, float seed) {
  float a[CH];
#pragma unroll
  for (int c = 0; c < CH; ++c) a[c] = seed * (c + 1);
  for (int it = 0; it < ITER; ++it) {
#pragma unroll
    for (int c = 0; c < CH; ++c) {
      int32_t t;
      asm volatile("cvt.rzi.s32.f32 %0, %1;" : "=r"(t) : "f"(a[c]));
      asm volatile("cvt.rn.f32.s32 %0, %1;" : "=f"(a[c]) : "r"(t));
    }
  }
  float s = 0;
#pragma unroll
  for (int c = 0; c < CH; ++c) s += a[c];
  if (s == 12345) out[threadIdx.x] = s;
}

template <typename F, typename... A>
void run(const char* name, F kern, int ops_per_iter, A... args) {
  int dev = 0, sms = 0, clk = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaDeviceGetAttribute(&clk, cudaDevAttrClockRate, dev);  // kHz
  const int blocks = sms * 8, threads = 256;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  for (int w = 0; w < 3; ++w) kern<<<blocks, threads>>>(args...);
  cudaEventRecord(e0);
  const int reps = 5;
  for (int r = 0; r < reps; ++r) kern<<<blocks, threads>>>(args...);
  cudaEventRecord(e1);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  const double ops = (double)reps * blocks * threads * ITER * CH * ops_per_iter;
  const double per_s = ops / (ms * 1e-3);
  const double per_clk_sm = per_s / (sms * (double)clk * 1e3);
  printf("%-14s %10.1f Gop/s  %7.1f lane-ops/clk/SM (at %d MHz nominal)  err=%s\n", name, per_s * 1e-9,
         per_clk_sm, clk / 1000, cudaGetErrorString(cudaGetLastError()));
}

int main() {
  void* buf;
  cudaMalloc(&buf, 1 << 16);
  run("ffma", k_ffma, 1, (float*)buf, 1.0001f);
  run("dfma", k_dfma, 1, (double*)buf, 1.0001);
  run("imad", k_imad, 1, (int32_t*)buf, 3);
  run("imad.hi", k_imadhi, 1, (uint32_t*)buf, 3u);
  run("imad.wide.s", k_imadwide, 1, (int64_t*)buf, 3);
  run("imad.wide.u", k_imadwideu, 1, (uint64_t*)buf, 3u);
  run("add", k_add, 1, (uint32_t*)buf, 3u);
  run("add64", k_add64, 1, (uint64_t*)buf, (uint64_t)3);
  run("shf", k_shf, 1, (uint32_t*)buf, 3u);
  run("clz+add", k_clz, 2, (uint32_t*)buf, 3u);
  run("cvt f64<->s64", k_cvt, 2, (double*)buf, 1.5);
  run("cvt f32<->s32", k_cvt32, 2, (float*)buf, 1.5f);
  cudaFree(buf);
  return 0;
}
