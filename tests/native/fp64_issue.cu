// Measurement of what one warp pays for FP64 work and memory on this GPU (the figures the SCIP-order node kernel
// is designed around).  One kernel, one block; every index stays inside the buffers allocated below.
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -o fp64_issue tests/native/fp64_issue.cu && ./fp64_issue
// Prints cycles per operation for: dependent DADD / DMUL / DFMA / DDIV chains; 8 independent DADD chains with 1..32
// lanes active and 1, 4 and 8 warps in the block; a double compare chain and the same compare on the integer bit
// patterns; a pointer chase through 4 KB (L1) and 4 MB (L2).
#include <cstdio>
#include <cuda_runtime.h>

__global__ void chains(double* out, long long* cyc, const int* chase, double y) {
  double x = 1.0 + threadIdx.x * 1e-9;
  long long t0, t1;
  const int N = 1024;
  t0 = clock64();
  for (int i = 0; i < N; ++i) x = x + y;
  t1 = clock64(); cyc[0] = t1 - t0;
  t0 = clock64();
  for (int i = 0; i < N; ++i) x = x * (1.0 + y);
  t1 = clock64(); cyc[1] = t1 - t0;
  t0 = clock64();
  for (int i = 0; i < N; ++i) x = fma(x, y, y);
  t1 = clock64(); cyc[2] = t1 - t0;
  double z = 3.0 + threadIdx.x;
  t0 = clock64();
  for (int i = 0; i < N / 8; ++i) z = y / z;
  t1 = clock64(); cyc[3] = (t1 - t0) * 8;
  x += z;
  int c = 0;
  t0 = clock64();
  for (int i = 0; i < N; ++i) { c += (x < y); x = __longlong_as_double(__double_as_longlong(x) ^ (long long)(c & 1)); }
  t1 = clock64(); cyc[4] = t1 - t0;
  long long xi = __double_as_longlong(x), yi = __double_as_longlong(y);
  t0 = clock64();
  for (int i = 0; i < N; ++i) { c += (xi < yi); xi ^= (c & 1); }
  t1 = clock64(); cyc[5] = t1 - t0;
  int p = 0;
  t0 = clock64();
  for (int i = 0; i < 256; ++i) p = chase[p];
  t1 = clock64(); cyc[6] = (t1 - t0) * 4;
  out[threadIdx.x] = x + c + (double)xi + p;
}

__global__ void independent(double* out, long long* cyc, int active, double y) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  double a0 = lane, a1 = lane + 1, a2 = lane + 2, a3 = lane + 3, a4 = lane + 4, a5 = lane + 5, a6 = lane + 6, a7 = lane + 7;
  __syncthreads();
  const long long t0 = clock64();
  if (lane < active)
    for (int i = 0; i < 512; ++i) { a0 += y; a1 += y; a2 += y; a3 += y; a4 += y; a5 += y; a6 += y; a7 += y; }
  __syncwarp();
  const long long t1 = clock64();
  if (lane == 0) cyc[warp] = t1 - t0;
  out[threadIdx.x] = a0 + a1 + a2 + a3 + a4 + a5 + a6 + a7;
}

static void setChase(int* d, int n) {  // one random cycle over n/32 lines, each entry the index of the next line
  int* h = new int[n]();
  const int m = n / 32;
  int* perm = new int[m];
  for (int i = 0; i < m; ++i) perm[i] = i;
  unsigned long long st = 12345;
  for (int i = m - 1; i > 0; --i) {
    st = st * 6364136223846793005ull + 1442695040888963407ull;
    const int j = (int)((st >> 33) % (unsigned long long)(i + 1));
    const int t = perm[i]; perm[i] = perm[j]; perm[j] = t;
  }
  for (int i = 0; i < m; ++i) h[perm[i] * 32] = perm[(i + 1) % m] * 32;
  cudaMemcpy(d, h, sizeof(int) * n, cudaMemcpyHostToDevice);
  delete[] h;
  delete[] perm;
}

int main() {
  double* out; long long* cyc; int* chase;
  const int big = 1 << 20;
  if (cudaMalloc(&out, 256 * sizeof(double)) || cudaMalloc(&cyc, 16 * sizeof(long long)) ||
      cudaMalloc(&chase, sizeof(int) * big)) { std::printf("allocation failed\n"); return 1; }
  const int sizes[2] = {1024, big};
  const char* where[2] = {"4 KB", "4 MB"};
  for (int k = 0; k < 2; ++k) {
    setChase(chase, sizes[k]);
    for (int rep = 0; rep < 2; ++rep) chains<<<1, 32>>>(out, cyc, chase, 1e-3);
    long long c[16];
    if (cudaMemcpy(c, cyc, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) { std::printf("kernel failed\n"); return 1; }
    if (k == 0)
      std::printf("dependent, cycles/op: dadd %.1f dmul %.1f dfma %.1f ddiv %.1f; compare chain: double %.1f, bit pattern %.1f\n",
                  c[0] / 1024.0, c[1] / 1024.0, c[2] / 1024.0, c[3] / 1024.0, c[4] / 1024.0, c[5] / 1024.0);
    std::printf("pointer chase through %s: %.1f cycles/load\n", where[k], c[6] / 1024.0);
  }
  const int acts[5] = {1, 2, 8, 16, 32}, warps[3] = {1, 4, 8};
  for (int w = 0; w < 3; ++w)
    for (int a = 0; a < 5; ++a) {
      for (int rep = 0; rep < 2; ++rep) independent<<<1, 32 * warps[w]>>>(out, cyc, acts[a], 1e-3);
      long long c[16];
      if (cudaMemcpy(c, cyc, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) { std::printf("kernel failed\n"); return 1; }
      std::printf("8 independent DADD chains, %d warp(s), %2d lane(s) active: %.1f cycles per DADD per warp\n", warps[w],
                  acts[a], c[0] / 4096.0);
    }
  return 0;
}
