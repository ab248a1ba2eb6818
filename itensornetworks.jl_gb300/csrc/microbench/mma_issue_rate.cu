// Cost of one tcgen05.mma (kind::f16, BF16 operands in shared memory, FP32
// accumulator in TMEM) as seen by the thread that issues it, for the shapes
// the tensor-core message kernel uses, with one to four concurrent issuers
// per SM (several CTAs per SM, or several issuing warps in one CTA).
//
// Every CTA zero-fills 48 KB of shared memory (A at [0, 16 KB), B at
// [16 KB, 48 KB), 128-byte swizzled, K-major), allocates `tcols` TMEM
// columns, and each issuing warp's lane 0 issues 256 MMAs into its own
// accumulator (columns [warp * N, warp * N + N)), commits, and waits (bounded)
// for completion; the second of two passes is timed with clock64.  Every
// descriptor stays inside its region and every accumulator inside the
// allocation.
//
// Build and run (sm_103a):
//   nvcc -gencode arch=compute_103a,code=sm_103a -O3 -std=c++17 -o mma_issue_rate mma_issue_rate.cu && ./mma_issue_rate
#include <cstdint>
#include <cstdio>

#include "../tc_ptx.cuh"

using namespace gbtn;

__global__ void mma_issue_probe(int M, int N, int issuers, int tcols, int nmma, long long* out, int* err) {
  extern __shared__ unsigned char sm_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(sm_raw) + 1023) & ~uintptr_t(1023));
  __shared__ uint32_t tslot;
  __shared__ __align__(8) uint64_t bar[4];
  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  for (int i = t; i < 49152 / 4; i += blockDim.x) reinterpret_cast<uint32_t*>(sm)[i] = 0;
  if (warp == 0) {
    tc::tmem_alloc(&tslot, tcols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    for (int i = 0; i < 4; ++i) tc::mbar_init(&bar[i], 1);
    tc::fence_mbar_init();
  }
  tc::fence_proxy_async_smem();
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = tslot;
  if (warp < issuers && lane == 0) {
    const uint64_t da = tc::smem_desc(tc::smem_u32(sm), 16, 1024);
    const uint64_t db = tc::smem_desc(tc::smem_u32(sm + 16384), 16, 1024);
    const uint32_t id = tc::idesc_bf16(M, N, 0, 0);
    const uint32_t col = (uint32_t)(warp * N);
    uint32_t par = 0;
    for (int rep = 0; rep < 2; ++rep) {
      const long long t0 = clock64();
      for (int i = 0; i < nmma; ++i) {
        const int kk = i & 3;  // K offset inside the 128-byte rows
        tc::mma_bf16(tmem + col, da + ((32 * kk) >> 4), db + ((32 * kk) >> 4), id, i > 0);
      }
      tc::mma_commit(&bar[warp]);
      if (!tc::mbar_wait(&bar[warp], par, 1000000000ull)) *err = 1;
      par ^= 1;
      if (rep == 1) out[blockIdx.x * 4 + warp] = clock64() - t0;
    }
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tmem, tcols);
}

int main() {
  int nsm = 0;
  cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, 0);
  const int max_blocks = 4 * nsm;
  long long* d_out = nullptr;
  int* d_err = nullptr;
  cudaMalloc(&d_out, sizeof(long long) * 4 * max_blocks);
  cudaMalloc(&d_err, sizeof(int));
  cudaMemset(d_err, 0, sizeof(int));
  const int smem = 49152 + 1024;
  cudaFuncSetAttribute(mma_issue_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
  const int nmma = 256;
  struct Run {
    int M, N, ctas_per_sm, issuers, tcols;
  } runs[] = {
      {128, 64, 1, 1, 512}, {128, 64, 2, 1, 256}, {128, 64, 4, 1, 128},  {64, 64, 1, 1, 512},
      {64, 64, 2, 1, 256},  {64, 64, 4, 1, 128},  {128, 256, 1, 1, 512}, {128, 256, 2, 1, 256},
      {128, 64, 1, 2, 512}, {128, 64, 1, 4, 512}, {64, 64, 1, 4, 512},   {128, 128, 1, 4, 512},
  };
  long long* h = new long long[4 * max_blocks];
  for (const Run& r : runs) {
    const int grid = nsm * r.ctas_per_sm;
    cudaMemset(d_out, 0, sizeof(long long) * 4 * max_blocks);
    mma_issue_probe<<<grid, 128, smem>>>(r.M, r.N, r.issuers, r.tcols, nmma, d_out, d_err);
    const cudaError_t e = cudaDeviceSynchronize();
    if (e != cudaSuccess) {
      printf("cuda error %s\n", cudaGetErrorString(e));
      return 1;
    }
    int herr = 0;
    cudaMemcpy(h, d_out, sizeof(long long) * 4 * grid, cudaMemcpyDeviceToHost);
    cudaMemcpy(&herr, d_err, sizeof(int), cudaMemcpyDeviceToHost);
    double sum = 0.0;
    int n = 0;
    for (int b = 0; b < grid; ++b)
      for (int w = 0; w < r.issuers; ++w) {
        sum += (double)h[b * 4 + w];
        ++n;
      }
    const double per = sum / n / nmma;                     // cycles per MMA seen by one issuer
    const double agg = per / (r.ctas_per_sm * r.issuers);  // cycles per MMA per SM
    printf("M%3d N%3d CTAs/SM %d issuers/CTA %d: %6.1f cycles/MMA per issuer, %6.1f per SM, %5.0f flop/cycle/SM%s\n",
           r.M, r.N, r.ctas_per_sm, r.issuers, per, agg, 2.0 * r.M * r.N * 16 / agg, herr ? "  TIMEOUT" : "");
  }
  delete[] h;
  return 0;
}
