// FP64 throughput probes of bench.py: the roofline denominators for the FP64 kernels (the measured-peaks file of
// this pool holds HBM and bf16 figures only). Not part of the library: bench.py compiles this file on its own
// (bench.build_probes) and loads it with ctypes.
//
//   bench_fp64_fma    independent register FMA chains (8 per thread, no memory traffic) on every SM, with
//                     `active_lanes` (1..32) lanes of every warp working: FP64 FMA throughput, and warp-level FP64
//                     instructions per second (equal rates for every lane count mean FP64 work is charged per warp
//                     instruction, whatever the number of active lanes)
//   bench_fp64_dmma   the same with the legacy FP64 tensor path, mma.sync .f64 (m8n8k4: 512 flops per warp
//                     instruction; m16n8k16: 4096), independent accumulators per warp: whether the FP64 MMA pipe
//                     beats the DFMA pipe for the small dense block updates of the LU and Gauss-Jordan kernels
//   bench_fp64_mixed  even warps run the DFMA chains, odd warps the m8n8k4 MMAs, with equal flops per warp: about
//                     the DFMA rate if the two share one FP64 unit, about twice it if they issue side by side
//
//   bench_exp         e^x throughput in register loops (8 blocks of 256 threads per SM, four independent sums per
//                     thread): 0 the loop alone, 1 CUDA's exp, 2 the library's table-driven tab_exp
//                     (spitfire_gb300/csrc/chem_device.cuh); the caller turns the times into FP64 instructions per call
//                     with the issue rate of bench_fp64_fma
//   bench_exp_values  both exponentials of n device values, for their accuracy against a wider reference
//
//   bench_store       stores from the SMs into a buffer, device memory or pinned host memory reached over the host
//                     link (the device address of a pinned allocation comes from cudaHostGetDevicePointer, and the
//                     call refuses host memory without one): pattern 0 coalesced (consecutive lanes, consecutive
//                     doubles), pattern 1 the thread-per-state Jacobian writer's (each lane fills its own 2916-double
//                     block sequentially, the 32 lanes of a warp 23 KB apart)
//
// Each FP64 launch covers 8 blocks of 256 threads per SM after a short warm-up launch, timed with CUDA events on the
// caller's stream (which the call synchronizes). Every loop is register-only with a fixed trip count, or, for the
// stores, bounded by the buffer size the caller passes.
#include <cuda_runtime.h>

#include <algorithm>

#include "spitfire_gb300/csrc/chem_device.cuh"

namespace {

__constant__ double cExpTab[128];  // sfgb::kExpTable, copied by exp_table_ready()

int exp_table_ready()
{
  static bool done = false;
  if (!done && cudaMemcpyToSymbol(cExpTab, sfgb::kExpTable, sizeof(sfgb::kExpTable)) == cudaSuccess) done = true;
  return done ? 0 : 1;
}

template <int WHICH>
__global__ void __launch_bounds__(256) exp_probe_kernel(int iters, double x0, double dx, double *sink)
{
  __shared__ __align__(16) double tab[128];
  if (threadIdx.x < 128) tab[threadIdx.x] = cExpTab[threadIdx.x];
  __syncthreads();
  double x = x0 - 40. * (double)((blockIdx.x * blockDim.x + threadIdx.x) & 1023) / 1024.;
  double a0 = 0., a1 = 0., a2 = 0., a3 = 0.;
  for (int i = 0; i < iters; ++i) {
    if (WHICH == 0) {
      a0 += x; a1 += x + dx; a2 += x + 2. * dx; a3 += x + 3. * dx;
    } else if (WHICH == 1) {
      a0 += exp(x); a1 += exp(x + dx); a2 += exp(x + 2. * dx); a3 += exp(x + 3. * dx);
    } else {
      a0 += sfgb::tab_exp(x, tab); a1 += sfgb::tab_exp(x + dx, tab);
      a2 += sfgb::tab_exp(x + 2. * dx, tab); a3 += sfgb::tab_exp(x + 3. * dx, tab);
    }
    x += 4. * dx;
  }
  const double v = a0 + a1 + a2 + a3;
  if (v == 12345.678) sink[0] = v;  // keeps the sums live
}

__global__ void exp_values_kernel(const double *x, double *oc, double *ot, long long n)
{
  __shared__ __align__(16) double tab[128];
  if (threadIdx.x < 128) tab[threadIdx.x] = cExpTab[threadIdx.x];
  __syncthreads();
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    oc[i] = exp(x[i]);
    ot[i] = sfgb::tab_exp(x[i], tab);
  }
}

__global__ void fma_probe_kernel(int iters, double seed, double *sink, int active_lanes)
{
  double a[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) a[k] = seed + k * 1e-3 + threadIdx.x * 1e-7;
  const double b = 0.999999999, c = 1e-9;
  if ((int)(threadIdx.x & 31) < active_lanes)
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
  double s = 0.;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += a[k];
  if (s == 12345.678) sink[0] = s;  // keeps the chains live
}

// m8n8k4: A one double per lane, B one, C/D two; eight independent accumulators per warp.
__global__ void dmma_m8n8k4_kernel(int iters, double seed, double *sink)
{
  const double a = 1e-3 * (seed + threadIdx.x * 1e-7), b = 1e-3 * (0.999 - threadIdx.x * 1e-9);
  double c[8][2];
#pragma unroll
  for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = k * 1e-6;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k)
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                   : "+d"(c[k][0]), "+d"(c[k][1])
                   : "d"(a), "d"(b));
  }
  double s = 0.;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
  if (s == 12345.678) sink[0] = s;
}

// m16n8k16: A eight doubles per lane, B four, C/D four; four independent accumulators per warp.
__global__ void dmma_m16n8k16_kernel(int iters, double seed, double *sink)
{
  const double a = 1e-4 * (seed + threadIdx.x * 1e-7), b = 1e-4 * (0.999 - threadIdx.x * 1e-9);
  double c[4][4];
#pragma unroll
  for (int k = 0; k < 4; ++k)
#pragma unroll
    for (int j = 0; j < 4; ++j) c[k][j] = (k + j) * 1e-6;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 4; ++k)
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, "
                   "{%4,%4,%4,%4,%4,%4,%4,%4}, {%5,%5,%5,%5}, {%0,%1,%2,%3};"
                   : "+d"(c[k][0]), "+d"(c[k][1]), "+d"(c[k][2]), "+d"(c[k][3])
                   : "d"(a), "d"(b));
  }
  double s = 0.;
#pragma unroll
  for (int k = 0; k < 4; ++k) s += c[k][0] + c[k][1] + c[k][2] + c[k][3];
  if (s == 12345.678) sink[0] = s;
}

// Even warps: 8 DFMA chains for 8*iters instructions (512 flops per warp per iteration); odd warps: 8 m8n8k4 MMAs
// every 8th iteration (4096 flops each time), the same flops per warp.
__global__ void mixed_probe_kernel(int iters, double seed, double *sink)
{
  double s = 0.;
  if (((threadIdx.x >> 5) & 1) == 0) {
    double a[8];
#pragma unroll
    for (int k = 0; k < 8; ++k) a[k] = seed + k * 1e-3 + threadIdx.x * 1e-7;
    const double b = 0.999999999, c = 1e-9;
    for (int i = 0; i < iters; ++i) {
#pragma unroll
      for (int k = 0; k < 8; ++k) a[k] = fma(a[k], b, c);
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) s += a[k];
  } else {
    const double a = 1e-3 * (seed + threadIdx.x * 1e-7), b = 1e-3 * (0.999 - threadIdx.x * 1e-9);
    double c[8][2];
#pragma unroll
    for (int k = 0; k < 8; ++k) c[k][0] = c[k][1] = k * 1e-6;
    for (int i = 0; i < iters / 8; ++i) {
#pragma unroll
      for (int k = 0; k < 8; ++k)
        asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};"
                     : "+d"(c[k][0]), "+d"(c[k][1])
                     : "d"(a), "d"(b));
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) s += c[k][0] + c[k][1];
  }
  if (s == 12345.678) sink[0] = s;
}

// pattern 0: grid-stride over doubles; pattern 1: lane-owned blocks of `block` doubles written in order.
__global__ void store_kernel(double *dst, long long n, int pattern, int block)
{
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const long long nt = (long long)gridDim.x * blockDim.x;
  if (pattern == 0) {
    for (long long i = tid; i < n; i += nt) dst[i] = (double)i;
  } else {
    const long long nblocks = n / block;
    for (long long b = tid; b < nblocks; b += nt) {
      double *o = dst + b * block;
      for (int k = 0; k < block; ++k) o[k] = (double)k;
    }
  }
}

template <class L>
int timed(cudaStream_t st, L launch, float *ms)
{
  launch(16);  // warm-up
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess) return 1;
  if (cudaEventCreate(&e1) != cudaSuccess) {
    cudaEventDestroy(e0);
    return 1;
  }
  cudaEventRecord(e0, st);
  launch(-1);
  cudaEventRecord(e1, st);
  cudaEventSynchronize(e1);
  cudaEventElapsedTime(ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

void shape(int *blocks, int *threads)
{
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  *blocks = nsm * 8;
  *threads = 256;
}

}  // namespace

extern "C" {

// TFLOP/s of the active lanes and warp-level FP64 instructions per second.
int bench_fp64_fma(int iters, int active_lanes, double *out_tflops, double *out_warp_instr_per_s, double *sink,
                   void *stream)
{
  if (iters < 1 || active_lanes < 1 || active_lanes > 32 || !out_tflops || !out_warp_instr_per_s || !sink) return 2;
  int blocks, threads;
  shape(&blocks, &threads);
  cudaStream_t st = (cudaStream_t)stream;
  float ms = 0.f;
  const int rc = timed(st, [&](int it) {
    fma_probe_kernel<<<blocks, threads, 0, st>>>(it < 0 ? iters : it, 1.0, sink, it < 0 ? active_lanes : 32);
  }, &ms);
  if (rc) return rc;
  const double warp_instr = 8.0 * (double)iters * blocks * (threads / 32);
  *out_warp_instr_per_s = warp_instr / (ms * 1e-3);
  *out_tflops = 2.0 * warp_instr * active_lanes / (ms * 1e-3) / 1e12;
  return 0;
}

// TFLOP/s of FP64 mma.sync, shape 0 = m8n8k4, 1 = m16n8k16.
int bench_fp64_dmma(int iters, int which, double *out_tflops, double *sink, void *stream)
{
  if (iters < 1 || (which != 0 && which != 1) || !out_tflops || !sink) return 2;
  int blocks, threads;
  shape(&blocks, &threads);
  cudaStream_t st = (cudaStream_t)stream;
  float ms = 0.f;
  const int rc = timed(st, [&](int it) {
    const int n = it < 0 ? iters : it;
    if (which == 0)
      dmma_m8n8k4_kernel<<<blocks, threads, 0, st>>>(n, 1.0, sink);
    else
      dmma_m16n8k16_kernel<<<blocks, threads, 0, st>>>(n, 1.0, sink);
  }, &ms);
  if (rc) return rc;
  const double per_instr = which == 0 ? 2.0 * 8 * 8 * 4 : 2.0 * 16 * 8 * 16;
  const double chains = which == 0 ? 8.0 : 4.0;
  const double flops = per_instr * chains * (double)iters * blocks * (threads / 32);
  *out_tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

// TFLOP/s of the mixed DFMA / MMA launch (iters a multiple of 8).
int bench_fp64_mixed(int iters, double *out_tflops, double *sink, void *stream)
{
  if (iters < 8 || iters % 8 || !out_tflops || !sink) return 2;
  int blocks, threads;
  shape(&blocks, &threads);
  cudaStream_t st = (cudaStream_t)stream;
  float ms = 0.f;
  const int rc = timed(st, [&](int it) {
    mixed_probe_kernel<<<blocks, threads, 0, st>>>(it < 0 ? iters : it, 1.0, sink);
  }, &ms);
  if (rc) return rc;
  const double flops = 512.0 * (double)iters * blocks * (threads / 32);
  *out_tflops = flops / (ms * 1e-3) / 1e12;
  return 0;
}

// Milliseconds of one exp_probe_kernel launch (4 iters exponentials per thread), which = 0, 1, 2 as above.
int bench_exp(int which, int iters, double *out_ms, double *sink, void *stream)
{
  if (which < 0 || which > 2 || iters < 1 || !out_ms || !sink) return 2;
  if (exp_table_ready()) return 1;
  int blocks, threads;
  shape(&blocks, &threads);
  cudaStream_t st = (cudaStream_t)stream;
  float ms = 0.f;
  const int rc = timed(st, [&](int it) {
    const int n = it < 0 ? iters : it;
    if (which == 0) exp_probe_kernel<0><<<blocks, threads, 0, st>>>(n, -1., 1.e-6, sink);
    if (which == 1) exp_probe_kernel<1><<<blocks, threads, 0, st>>>(n, -1., 1.e-6, sink);
    if (which == 2) exp_probe_kernel<2><<<blocks, threads, 0, st>>>(n, -1., 1.e-6, sink);
  }, &ms);
  *out_ms = ms;
  return rc;
}

// exp (CUDA) and tab_exp of n device values into two device arrays.
int bench_exp_values(const double *x, double *out_cuda, double *out_tab, long long n, void *stream)
{
  if (!x || !out_cuda || !out_tab || n < 0) return 2;
  if (n == 0) return 0;
  if (exp_table_ready()) return 1;
  int blocks, threads;
  shape(&blocks, &threads);
  exp_values_kernel<<<blocks, threads, 0, (cudaStream_t)stream>>>(x, out_cuda, out_tab, n);
  return cudaGetLastError() == cudaSuccess ? 0 : 1;
}

// GB/s of stores into `buffer` (bytes, a device allocation or a pinned host allocation).
int bench_store(void *buffer, long long bytes, int pattern, double *out_gbs, void *stream)
{
  if (!buffer || bytes < 8 || (pattern != 0 && pattern != 1) || !out_gbs) return 2;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, buffer) != cudaSuccess) return 3;
  double *dst = nullptr;
  if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) {
    dst = static_cast<double *>(buffer);
  } else if (attr.type == cudaMemoryTypeHost) {
    void *d = nullptr;
    if (cudaHostGetDevicePointer(&d, buffer, 0) != cudaSuccess || !d) return 4;
    dst = static_cast<double *>(d);
  } else {
    return 5;  // pageable host memory: not written from the device here
  }
  const int block = 2916;
  const long long n = pattern == 0 ? bytes / 8 : (bytes / 8 / block) * block;
  int dev = 0, nsm = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev);
  cudaStream_t st = (cudaStream_t)stream;
  // pattern 1: one lane per block, 8 resident warps of 4-warp blocks per SM, as the Jacobian kernel runs
  const int threads = pattern == 0 ? 256 : 128;
  const int blocks = pattern == 0 ? nsm * 8 : nsm * 2;
  float ms = 0.f;
  const int rc = timed(st, [&](int it) {
    store_kernel<<<blocks, threads, 0, st>>>(dst, it < 0 ? n : std::min<long long>(n, (long long)block * 64),
                                             pattern, block);
  }, &ms);
  if (rc) return rc;
  *out_gbs = (double)n * 8 / (ms * 1e-3) / 1e9;
  return 0;
}

}  // extern "C"
