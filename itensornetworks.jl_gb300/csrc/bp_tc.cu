// BF16 tensor-core (tcgen05) message kernel for degree-4 vertices with d = 2
// and chi = 8 on every leg -- the interior of a square PEPS at the target bond
// dimension, which carries ~95 % of the flops of a 32x32 chi=8 sweep.
//
// Split the site tensor by its site index s into two 64 x 64 matrices
//   Z_s[c2][c1],  c1 = l1 + 8 l2,  c2 = l3 + 8 l4
// (A[s, l1..l4] = Z_s[c2][c1]).  Stacked, Z is a 128 x 64 BF16 matrix kept in
// shared memory in the 128-byte-swizzled layout, which the tensor core reads
// both as a K-major operand (rows (s,c2), K = c1) and, through the symmetry of
// the swizzle atom, as an MN-major operand (M = (s,c1), K = c2).  With the
// Kronecker products K12 = M1 (x) M2 and K34 = M3 (x) M4 of the incoming
// messages (bra x ket):
//   GEMM1   T12[(s,c2), (b1,b2)] = sum_c1 Z[(s,c2), c1] K12[(b1,b2), c1]       M=128 N=64  K=64
//   GEMM1'  T34[(s,c1), (b3,b4)] = sum_c2 Z_s[c2][c1]  K34[(b3,b4), c2]        M=128 N=64  K=64
//   GEMM2   D2[(s,c2), (s',c2')] = sum_c1' T12[(s,c2), c1'] Z_s'[c2'][c1']     M=128 N=128 K=64
//   GEMM2'  D2'[(s,c1),(s',c1')] = sum_c2' T34[(s,c1), c2'] Z_s'[c2'][c1']     M=128 N=128 K=64
// The s = s' diagonal blocks summed over s give the two-leg environments
// G34[(a3,a4),(b3,b4)] and G12[(a1,a2),(b1,b2)] (ket x bra), from which
//   out3[b3,a3] = sum G34[(a3,a4),(b3,b4)] M4[b4,a4],  out4 likewise with M3,
//   out1[b1,a1] = sum G12[(a1,a2),(b1,b2)] M2[b2,a2],  out2 likewise with M1
// are 64 x 64 x 64 FP32 contractions on the CUDA cores.  Outputs are
// normalised in FP64 and written as FP32 messages (updated_message,
// src/caches/abstractbeliefpropagationcache.jl:225-239).
//
// Per vertex: one 16 KB TMA bulk copy of the pre-swizzled BF16 image of Z
// (double-buffered, prefetched one vertex ahead), 16 tcgen05.mma instructions
// with FP32 accumulation in TMEM (256 columns), 8 tcgen05.ld per thread.
// 128 threads per CTA, 2 CTAs per SM, persistent over the vertex list.
#include <cuda_bf16.h>

#include "gbtn_internal.h"
#include "tc_ptx.cuh"

namespace gbtn {
namespace {

constexpr int kTcThreads = 128;
constexpr uint32_t kZElems = 8192;
constexpr uint32_t kZBytes = kZElems * 2;
constexpr uint64_t kWaitNs = 1000000000ull;  // 1 s bound on every wait

// shared-memory carve-up (bytes from a 1024-aligned base)
constexpr int kOffZ0 = 0, kOffZ1 = 16384, kOffT12 = 32768, kOffT34 = 49152, kOffK12 = 65536, kOffK34 = 73728;
constexpr int kGStride = 65;  // padded FP32 row of the 64 x 64 environment
constexpr int kOffG = 81920;
constexpr int kOffMsg = kOffG + 64 * kGStride * 4;  // 4 x 64 FP32 incoming messages
constexpr int kOffRes = kOffMsg + 4 * 64 * 4;       // 4 x 64 FP32 outgoing messages
constexpr int kOffBar = kOffRes + 4 * 64 * 4;       // mma bar, 2 TMA bars
constexpr int kOffTmem = kOffBar + 3 * 8;
constexpr int kOffFlag = kOffTmem + 4;
constexpr int kSmemUsed = kOffFlag + 4;
constexpr int kSmemBytes = kSmemUsed + 1024;  // room to align the base
constexpr uint32_t kTmemCols = 256;

constexpr uint32_t kIdescG1 = tc::idesc_bf16(128, 64, 0, 0);
constexpr uint32_t kIdescG1mn = tc::idesc_bf16(128, 64, 1, 0);
constexpr uint32_t kIdescG2 = tc::idesc_bf16(128, 128, 0, 0);
constexpr uint32_t kIdescG2mn = tc::idesc_bf16(128, 128, 0, 1);

__device__ __forceinline__ double tc_warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Write 64 FP32 values as one 128-byte BF16 row of a 128B-swizzled tile.
__device__ __forceinline__ void store_row_swizzled(__nv_bfloat16* tile, int row, const float (&v)[64]) {
  uint4* base = reinterpret_cast<uint4*>(tile + row * 64);
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    __nv_bfloat162 p0 = __floats2bfloat162_rn(v[8 * j + 0], v[8 * j + 1]);
    __nv_bfloat162 p1 = __floats2bfloat162_rn(v[8 * j + 2], v[8 * j + 3]);
    __nv_bfloat162 p2 = __floats2bfloat162_rn(v[8 * j + 4], v[8 * j + 5]);
    __nv_bfloat162 p3 = __floats2bfloat162_rn(v[8 * j + 6], v[8 * j + 7]);
    uint4 q;
    q.x = *reinterpret_cast<uint32_t*>(&p0);
    q.y = *reinterpret_cast<uint32_t*>(&p1);
    q.z = *reinterpret_cast<uint32_t*>(&p2);
    q.w = *reinterpret_cast<uint32_t*>(&p3);
    base[j ^ (row & 7)] = q;
  }
}

// FP64 normalisation, FP32 store and message diff of one 8 x 8 message by one warp.
__device__ __forceinline__ double tc_finalize(const float* res, const float* old, float* out, int normalize,
                                              bool want_diff, int lane) {
  const double v0 = res[lane], v1 = res[lane + 32];
  const double nrm2 = tc_warp_sum(v0 * v0 + v1 * v1);
  const double sc = (normalize && nrm2 > 0.0) ? 1.0 / sqrt(nrm2) : 1.0;
  const float n0 = (float)(v0 * sc), n1 = (float)(v1 * sc);
  double o0 = 0.0, o1 = 0.0;
  if (want_diff) {
    o0 = old[lane];
    o1 = old[lane + 32];
  }
  __syncwarp();
  out[lane] = n0;
  out[lane + 32] = n1;
  double diff = 0.0;
  if (want_diff) {
    const double a0 = n0, a1 = n1;
    const double dot = tc_warp_sum(a0 * o0 + a1 * o1);
    const double na = tc_warp_sum(a0 * a0 + a1 * a1);
    const double nb = tc_warp_sum(o0 * o0 + o1 * o1);
    diff = 1.0 - (dot * dot) / (na * nb);
  }
  return diff;
}

}  // namespace

// One CTA walks work[blockIdx.x], work[blockIdx.x + gridDim.x], ...; vertex v
// reads its Z image at zimg + vslot[v] * 8192.  err (device) receives
// GBTN_ERR_TIMEOUT when a bounded wait gives up; the CTA then drains its own
// copies in flight, frees its TMEM and returns.
__global__ void __launch_bounds__(kTcThreads, 2)
    tc_vertex_kernel(const int* __restrict__ work, int nwork, const int* __restrict__ vslot,
                     const VDesc* __restrict__ vd, const __nv_bfloat16* __restrict__ zimg, const float* msg_in,
                     float* msg_out, const long long* __restrict__ msg_off, double* diffs, const int* converged,
                     int normalize, int want_diff, int* err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  __nv_bfloat16* Zbuf[2] = {reinterpret_cast<__nv_bfloat16*>(sm + kOffZ0),
                            reinterpret_cast<__nv_bfloat16*>(sm + kOffZ1)};
  __nv_bfloat16* T12 = reinterpret_cast<__nv_bfloat16*>(sm + kOffT12);
  __nv_bfloat16* T34 = reinterpret_cast<__nv_bfloat16*>(sm + kOffT34);
  __nv_bfloat16* K12 = reinterpret_cast<__nv_bfloat16*>(sm + kOffK12);
  __nv_bfloat16* K34 = reinterpret_cast<__nv_bfloat16*>(sm + kOffK34);
  float* G = reinterpret_cast<float*>(sm + kOffG);
  float* MSG = reinterpret_cast<float*>(sm + kOffMsg);
  float* RES = reinterpret_cast<float*>(sm + kOffRes);
  uint64_t* mma_bar = reinterpret_cast<uint64_t*>(sm + kOffBar);
  uint64_t* tma_bar = mma_bar + 1;  // [2]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kOffTmem);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(sm + kOffFlag);

  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(mma_bar, 1);
    tc::mbar_init(&tma_bar[0], 1);
    tc::mbar_init(&tma_bar[1], 1);
    tc::fence_mbar_init();
    *abort_flag = 0;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t lane_base = (uint32_t)(32 * warp) << 16;

  // thread-0 bookkeeping of the asynchronous work in flight
  uint32_t mma_phase = 0, tma_phase0 = 0, tma_phase1 = 0;
  int tma_pending0 = 0, tma_pending1 = 0, mma_pending = 0;

  auto issue_z = [&](int w, int b) {
    uint64_t* bar = &tma_bar[b];
    tc::mbar_expect_tx(bar, kZBytes);
    tc::tma_load_1d(Zbuf[b], zimg + (size_t)vslot[work[w]] * kZElems, kZBytes, bar);
    if (b == 0) tma_pending0 = 1; else tma_pending1 = 1;
  };
  // thread 0: wait for buffer b's copy; returns false on timeout
  auto wait_z = [&](int b) -> bool {
    const bool ok = tc::mbar_wait(&tma_bar[b], b == 0 ? tma_phase0 : tma_phase1, kWaitNs);
    if (ok) {
      if (b == 0) { tma_phase0 ^= 1; tma_pending0 = 0; } else { tma_phase1 ^= 1; tma_pending1 = 0; }
    }
    return ok;
  };
  auto wait_mma = [&]() -> bool {
    const bool ok = tc::mbar_wait(mma_bar, mma_phase, kWaitNs);
    if (ok) { mma_phase ^= 1; mma_pending = 0; }
    return ok;
  };

  int w = blockIdx.x;
  if (t == 0 && w < nwork) issue_z(w, 0);
  for (int i = 0; w < nwork; ++i, w += gridDim.x) {
    const int buf = i & 1;
    const int v = work[w];
    const int wn = w + gridDim.x;
    if (t == 0 && wn < nwork) issue_z(wn, buf ^ 1);  // buffer buf^1 is idle: its MMAs completed last iteration
    const VDesc& dv = vd[v];
    const bool skip = converged && converged[dv.net];
    for (int q = t; q < 256; q += kTcThreads) {
      const int p = q >> 6, e = q & 63;
      const long long off = msg_off[skip ? dv.out_de[p] : dv.in_de[p]];
      if (skip)
        msg_out[off + e] = msg_in[off + e];
      else
        MSG[q] = msg_in[off + e];
    }
    __syncthreads();
    if (!skip) {
      // Kronecker products K12 = M1 (x) M2 (threads 0-63) and K34 = M3 (x) M4 (64-127):
      // row n = b_a + 8 b_b, column k = a_a + 8 a_b, value M_a[b_a, a_a] M_b[b_b, a_b].
      const int n = t & 63;
      const float* Ma = MSG + (t < 64 ? 0 : 128);
      const float* Mb = Ma + 64;
      const int ba = n & 7, bb = n >> 3;
      float row[64];
#pragma unroll
      for (int ab = 0; ab < 8; ++ab) {
        const float mb = Mb[bb + 8 * ab];
#pragma unroll
        for (int aa = 0; aa < 8; ++aa) row[aa + 8 * ab] = Ma[ba + 8 * aa] * mb;
      }
      store_row_swizzled(t < 64 ? K12 : K34, n, row);
      tc::fence_proxy_async_smem();
    }
    if (t == 0) *abort_flag = wait_z(buf) ? 0 : 1;
    __syncthreads();
    if (*abort_flag) break;
    if (skip) continue;

    // ---- GEMM1 / GEMM1' ----
    const uint32_t zaddr = tc::smem_u32(Zbuf[buf]);
    if (t == 0) {
      tc::tc_fence_after();
      const uint32_t k12 = tc::smem_u32(K12), k34 = tc::smem_u32(K34);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(tmem + 0, tc::smem_desc(zaddr + 32 * kk, 16, 1024), tc::smem_desc(k12 + 32 * kk, 16, 1024),
                     kIdescG1, kk > 0);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(tmem + 64, tc::smem_desc(zaddr + 2048 * kk, 8192, 1024),
                     tc::smem_desc(k34 + 32 * kk, 16, 1024), kIdescG1mn, kk > 0);
      tc::mma_commit(mma_bar);
      mma_pending = 1;
      *abort_flag = wait_mma() ? 0 : 1;
    }
    __syncthreads();
    if (*abort_flag) break;
    tc::tc_fence_after();
    {
      float d[64];
      tc::tmem_ld_x64(tmem + lane_base + 0, d);
      store_row_swizzled(T12, t, d);
      tc::tmem_ld_x64(tmem + lane_base + 64, d);
      store_row_swizzled(T34, t, d);
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();

    // ---- GEMM2 / GEMM2' ----
    if (t == 0) {
      tc::tc_fence_after();
      const uint32_t t12 = tc::smem_u32(T12), t34 = tc::smem_u32(T34);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(tmem + 0, tc::smem_desc(t12 + 32 * kk, 16, 1024), tc::smem_desc(zaddr + 32 * kk, 16, 1024),
                     kIdescG2, kk > 0);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(tmem + 128, tc::smem_desc(t34 + 32 * kk, 16, 1024),
                     tc::smem_desc(zaddr + 2048 * kk, 8192, 1024), kIdescG2mn, kk > 0);
      tc::mma_commit(mma_bar);
      mma_pending = 1;
      *abort_flag = wait_mma() ? 0 : 1;
    }
    __syncthreads();
    if (*abort_flag) break;
    tc::tc_fence_after();

    // ---- two-leg environments and the four outgoing messages ----
    const int s = warp >> 1, c = t & 63;
    const float* M1 = MSG;
    const float* M2 = MSG + 64;
    const float* M3 = MSG + 128;
    const float* M4 = MSG + 192;
    for (int half = 0; half < 2; ++half) {
      float d[64];
      tc::tmem_ld_x64(tmem + lane_base + 128 * half + 64 * s, d);
      if (s == 0) {
#pragma unroll
        for (int j = 0; j < 64; ++j) G[c * kGStride + j] = d[j];
      }
      __syncthreads();
      if (s == 1) {
#pragma unroll
        for (int j = 0; j < 64; ++j) G[c * kGStride + j] += d[j];
      }
      __syncthreads();
      // half 0: G = G34 -> out3 (t < 64, uses M4) and out4 (t >= 64, uses M3)
      // half 1: G = G12 -> out1 (t < 64, uses M2) and out2 (t >= 64, uses M1)
      const int u = t & 63, bx = u & 7, ax = u >> 3;
      float acc = 0.f;
      if (t < 64) {
        const float* Mo = half == 0 ? M4 : M2;  // other leg of the pair, contracted
#pragma unroll
        for (int ay = 0; ay < 8; ++ay)
#pragma unroll
          for (int by = 0; by < 8; ++by) acc = fmaf(G[(ax + 8 * ay) * kGStride + bx + 8 * by], Mo[by + 8 * ay], acc);
        RES[(half == 0 ? 2 : 0) * 64 + u] = acc;
      } else {
        const float* Mo = half == 0 ? M3 : M1;
#pragma unroll
        for (int ay = 0; ay < 8; ++ay)
#pragma unroll
          for (int by = 0; by < 8; ++by) acc = fmaf(G[(ay + 8 * ax) * kGStride + by + 8 * bx], Mo[by + 8 * ay], acc);
        RES[(half == 0 ? 3 : 1) * 64 + u] = acc;
      }
      __syncthreads();
    }
    tc::tc_fence_before();
    // warp p finalises the message leaving on leg p
    {
      const int de = dv.out_de[warp];
      const long long off = msg_off[de];
      const double df = tc_finalize(RES + 64 * warp, msg_in + off, msg_out + off, normalize, want_diff != 0, lane);
      if (want_diff && lane == 0) diffs[de] = df;
    }
  }

  // drain: after a timeout, wait (bounded) for this CTA's own copies and MMAs
  if (t == 0 && *abort_flag) {
    atomicExch(err, (int)GBTN_ERR_TIMEOUT);
    if (tma_pending0) wait_z(0);
    if (tma_pending1) wait_z(1);
    if (mma_pending) wait_mma();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

// Swizzled BF16 image of Z for every slot: element A[s, c1, c2] (idx = s + 2 c1
// + 128 c2) goes to row r = 64 s + c2, 16-byte chunk (c1 / 8) ^ (r % 8).
__global__ void build_zimg_kernel(const int* __restrict__ slot_vertex, int nslot, const VDesc* __restrict__ vd,
                                  const double* __restrict__ fac, __nv_bfloat16* __restrict__ zimg) {
  const int slot = blockIdx.x;
  if (slot >= nslot) return;
  const double* a = fac + vd[slot_vertex[slot]].a_off;
  __nv_bfloat16* z = zimg + (size_t)slot * kZElems;
  for (int idx = threadIdx.x; idx < (int)kZElems; idx += blockDim.x) {
    const int s = idx & 1, c1 = (idx >> 1) & 63, c2 = idx >> 7;
    const int r = 64 * s + c2;
    z[r * 64 + (((c1 >> 3) ^ (r & 7)) << 3) + (c1 & 7)] = __double2bfloat16(a[idx]);
  }
}

}  // namespace gbtn

namespace gbtn {

bool tc_eligible(const VDesc& d) {
  if (d.k != 4 || d.d != 2) return false;
  for (int p = 0; p < 4; ++p)
    if (d.chi[p] != 8) return false;
  return true;
}

void launch_build_zimg(const int* slot_vertex, int nslot, const VDesc* vd, const double* fac, __nv_bfloat16* zimg,
                       cudaStream_t s) {
  if (nslot == 0) return;
  build_zimg_kernel<<<nslot, 256, 0, s>>>(slot_vertex, nslot, vd, fac, zimg);
  GBTN_CUDA(cudaGetLastError());
}

void launch_tc_vertices(const int* work, int nwork, const int* vslot, const VDesc* vd, const __nv_bfloat16* zimg,
                        const float* msg_in, float* msg_out, const long long* msg_off, double* diffs,
                        const int* converged, int normalize, int want_diff, int* err, cudaStream_t s) {
  if (nwork == 0) return;
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0;
    GBTN_CUDA(cudaGetDevice(&dev));
    GBTN_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  GBTN_CUDA(cudaFuncSetAttribute(tc_vertex_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
  const int grid = nwork < 2 * nsm ? nwork : 2 * nsm;
  tc_vertex_kernel<<<grid, kTcThreads, kSmemBytes, s>>>(work, nwork, vslot, vd, zimg, msg_in, msg_out, msg_off,
                                                         diffs, converged, normalize, want_diff, err);
  GBTN_CUDA(cudaGetLastError());
}

}  // namespace gbtn
