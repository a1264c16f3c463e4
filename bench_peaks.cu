// Peak probes for the roofline denominators that the measured HBM-copy and bf16-GEMM figures
// do not cover on this part: DFMA, FP64 mma.sync (m8n8k4 and m16n8k16), FFMA, and
// pinned / pageable host<->device copy bandwidth. Built and run by
// `python bench.py --workload peaks`. Every kernel runs a fixed iteration count of
// independent FMA chains and writes only out[gid].
#include <cstdio>
#include <cuda_runtime.h>

#define CK(x) do { cudaError_t e = (x); if (e != cudaSuccess) { printf("ERR %s at %d: %s\n", #x, __LINE__, cudaGetErrorString(e)); return 1; } } while (0)

__global__ void dfma_k(double* out, int iters) {
  double a[8];
  for (int j = 0; j < 8; j++) a[j] = threadIdx.x * 1e-3 + j;
  const double b = 0.999999, c = 1e-7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++) a[j] = fma(a[j], b, c);
  }
  double s = 0; for (int j = 0; j < 8; j++) s += a[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void ffma_k(float* out, int iters) {
  float a[16];
  for (int j = 0; j < 16; j++) a[j] = threadIdx.x * 1e-3f + j;
  const float b = 0.999999f, c = 1e-7f;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 16; j++) a[j] = fmaf(a[j], b, c);
  }
  float s = 0; for (int j = 0; j < 16; j++) s += a[j];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void dmma884_k(double* out, int iters) {
  double a = 1e-3 * threadIdx.x, b = 0.5;
  double c[8][2];
  for (int j = 0; j < 8; j++) { c[j][0] = j; c[j][1] = -j; }
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 8; j++) {
      asm volatile("mma.sync.aligned.m8n8k4.row.col.f64.f64.f64.f64 {%0,%1}, {%2}, {%3}, {%0,%1};\n"
                   : "+d"(c[j][0]), "+d"(c[j][1]) : "d"(a), "d"(b));
    }
  }
  double s = 0; for (int j = 0; j < 8; j++) s += c[j][0] + c[j][1];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

__global__ void dmma16816_k(double* out, int iters) {
  double a[8], b[4];
  for (int j = 0; j < 8; j++) a[j] = 1e-3 * (threadIdx.x + j);
  for (int j = 0; j < 4; j++) b[j] = 0.25 * j;
  double c[4][4];
  for (int j = 0; j < 4; j++) for (int k = 0; k < 4; k++) c[j][k] = j - k;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
      asm volatile("mma.sync.aligned.m16n8k16.row.col.f64.f64.f64.f64 {%0,%1,%2,%3}, {%4,%5,%6,%7,%8,%9,%10,%11}, {%12,%13,%14,%15}, {%0,%1,%2,%3};\n"
                   : "+d"(c[j][0]), "+d"(c[j][1]), "+d"(c[j][2]), "+d"(c[j][3])
                   : "d"(a[0]), "d"(a[1]), "d"(a[2]), "d"(a[3]), "d"(a[4]), "d"(a[5]), "d"(a[6]), "d"(a[7]),
                     "d"(b[0]), "d"(b[1]), "d"(b[2]), "d"(b[3]));
    }
  }
  double s = 0; for (int j = 0; j < 4; j++) for (int k = 0; k < 4; k++) s += c[j][k];
  out[blockIdx.x * blockDim.x + threadIdx.x] = s;
}

template <class F>
float timeit(F f) {
  cudaEvent_t e0, e1; cudaEventCreate(&e0); cudaEventCreate(&e1);
  f();  // warm
  cudaDeviceSynchronize();
  cudaEventRecord(e0); f(); cudaEventRecord(e1); cudaEventSynchronize(e1);
  float ms; cudaEventElapsedTime(&ms, e0, e1);
  return ms;
}

int main() {
  cudaDeviceProp p; CK(cudaGetDeviceProperties(&p, 0));
  printf("dev %s sm %d.%d SMs %d smemOptin %zu L2 %d\n", p.name, p.major, p.minor, p.multiProcessorCount,
         p.sharedMemPerBlockOptin, p.l2CacheSize);
  int nsm = p.multiProcessorCount;
  int blocks = nsm * 8, threads = 256;
  size_t nthr = (size_t)blocks * threads;
  double* dout; CK(cudaMalloc(&dout, nthr * sizeof(double)));
  float* fout; CK(cudaMalloc(&fout, nthr * sizeof(float)));
  int it = 4096;
  float ms = timeit([&] { dfma_k<<<blocks, threads>>>(dout, it); });
  CK(cudaGetLastError());
  printf("DFMA   %.3f ms  %.2f TFLOP/s\n", ms, 2.0 * 8 * it * nthr / ms / 1e9);
  it = 16384;
  ms = timeit([&] { ffma_k<<<blocks, threads>>>(fout, it); });
  CK(cudaGetLastError());
  printf("FFMA   %.3f ms  %.2f TFLOP/s\n", ms, 2.0 * 16 * it * nthr / ms / 1e9);
  it = 1024;
  ms = timeit([&] { dmma884_k<<<blocks, threads>>>(dout, it); });
  CK(cudaGetLastError());
  printf("DMMA884 %.3f ms  %.2f TFLOP/s\n", ms, 512.0 * 8 * it * (nthr / 32) / ms / 1e9);
  it = 256;
  ms = timeit([&] { dmma16816_k<<<blocks, threads>>>(dout, it); });
  CK(cudaGetLastError());
  printf("DMMA16816 %.3f ms  %.2f TFLOP/s\n", ms, 2.0 * 16 * 8 * 16 * 4 * it * (nthr / 32) / ms / 1e9);
  // H2D / D2H pinned bandwidth
  size_t nb = (size_t)1 << 30;
  void *h, *d; CK(cudaMallocHost(&h, nb)); CK(cudaMalloc(&d, nb));
  ms = timeit([&] { cudaMemcpy(d, h, nb, cudaMemcpyHostToDevice); });
  printf("H2D pinned 1GiB %.3f ms %.1f GB/s\n", ms, nb / ms / 1e6);
  ms = timeit([&] { cudaMemcpy(h, d, nb, cudaMemcpyDeviceToHost); });
  printf("D2H pinned 1GiB %.3f ms %.1f GB/s\n", ms, nb / ms / 1e6);
  void* hp = malloc(nb);
  for (size_t i = 0; i < nb; i += 4096) ((char*)hp)[i] = 1;
  ms = timeit([&] { cudaMemcpy(d, hp, nb, cudaMemcpyHostToDevice); });
  printf("H2D pageable 1GiB %.3f ms %.1f GB/s\n", ms, nb / ms / 1e6);
  free(hp);
  cudaFreeHost(h); cudaFree(d); cudaFree(dout); cudaFree(fout);
  return 0;
}
