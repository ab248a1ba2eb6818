// BF16 tensor-core (tcgen05) message kernel for degree-4 vertices with d = 2
// and chi = 8 on every leg -- the interior of a square PEPS at the target bond
// dimension, which carries ~95 % of the flops of a 32x32 chi=8 sweep.
//
// Split the site tensor by its site index s into two 64 x 64 matrices
//   Z_s[c2][c1],  c1 = l1 + 8 l2,  c2 = l3 + 8 l4
// (A[s, l1..l4] = Z_s[c2][c1]).  Stacked, Z is a 128 x 64 BF16 matrix kept in
// shared memory in the 128-byte-swizzled layout, which the tensor core reads
// both as a K-major operand (rows (s,c2), K = c1) and, through the symmetry of
// the swizzle atom, as an MN-major operand (M or N = c1, K = (s,c2)).  With the
// Kronecker products K12 = M1 (x) M2 and K34 = M3 (x) M4 of the incoming
// messages (bra x ket):
//   GEMM1   T12[(s,c2), (b1,b2)] = sum_c1 Z[(s,c2), c1] K12[(b1,b2), c1]          M=128 N=64 K=64
//   GEMM1'  T34[(s,c1), (b3,b4)] = sum_c2 Z_s[c2][c1] K34[(b3,b4), c2]            M=128 N=64 K=64
//   GEMM2   G34[c2, c2']  = sum_{s,c1'} T12[(s,c2), c1'] Z_s[c2'][c1']             M=64  N=64 K=128
//   GEMM2'  G12[c1, c1']  = sum_{s,c2'} T34[(s,c1), c2'] Z_s[c2'][c1']             M=64  N=64 K=128
// G34[(a3,a4),(b3,b4)] and G12[(a1,a2),(b1,b2)] are the two-leg environments
// (ket x bra); the outgoing messages
//   out3[b3,a3] = sum G34[(a3,a4),(b3,b4)] M4[b4,a4],  out4[b4,a4] = sum G34 M3[b3,a3],
//   out1[b1,a1] = sum G12[(a1,a2),(b1,b2)] M2[b2,a2],  out2[b2,a2] = sum G12 M1[b1,a1]
// are FP32 contractions done from registers (warp shuffles plus one
// cross-warp sum).  Each message is normalised and written as FP32
// (updated_message, src/caches/abstractbeliefpropagationcache.jl:225-239).
// BP is invariant under message scaling, so this reduced-precision phase
// normalises in FP32; the FP64 refinement sweeps that follow normalise in FP64.
//
// A vertex with fewer legs or smaller bond dimensions (d = 2, degree <= 4,
// chi <= 8) runs the same kernel zero-padded: its image holds zeros beyond
// each chi, a missing leg has dimension 1 and receives the 1 x 1 message 1,
// compact chi x chi messages are gathered into the 8 x 8 layout and scattered
// back.  Every product with a padding entry is an exact zero, so norms and
// message_diff are those of the compact messages.
//
// Per vertex: one 16 KB TMA bulk copy of the pre-swizzled BF16 image of Z,
// 24 tcgen05.mma instructions (4.2 MFLOP) accumulating in FP32 in TMEM (128
// columns: D1 | D1', then G34 | G12) issued by two threads (one per
// accumulator chain), two MMA round trips, seven CTA barriers,
// 128 threads.  Four CTAs share an SM (53 KB of shared memory each; the
// Kronecker products and then T12 share one region), the next vertex's Z is
// copied while the current one finishes and its messages are loaded into
// registers ahead of use.
#include <cuda_bf16.h>

#include "gbtn_internal.h"
#include "tc_ptx.cuh"

namespace gbtn {
namespace {

constexpr int kTcThreads = 128;
constexpr int kTcBlocksPerSm = 4;
constexpr uint32_t kZElems = 8192;
constexpr uint32_t kZBytes = kZElems * 2;
constexpr uint64_t kWaitNs = 1000000000ull;  // 1 s bound on every wait

// Failure-detection test (gbtn_ctx_test_wait_timeout): bytes added to the
// transaction count each image copy's mbarrier expects, passed to every
// launch.  Nonzero, the copy lands but the barrier never completes, so the
// bounded wait gives up and the sweep reports a timeout; 0 in normal use.
unsigned int g_tc_test_extra_tx = 0;

// shared-memory carve-up (bytes from a 1024-aligned base)
constexpr int kOffZ = 0;           // 16 KB: Z image (TMA destination)
constexpr int kOffKT = 16384;      // K12 | K34 (2 x 8 KB), then T12 as two 8 KB tiles (s = 0, 1)
constexpr int kOffT34 = 32768;     // T34 as two 8 KB tiles (s = 0, 1)
constexpr int kOffPart = 49152;    // cross-warp partial sums: 2 pairs x 4 warps x 64 FP32
constexpr int kOffMsg = kOffPart + 2048;  // 4 x 64 FP32 incoming messages
constexpr int kOffRes = kOffMsg + 1024;   // 4 x 64 FP32 outgoing messages
constexpr int kOffRec = kOffRes + 1024;   // 3 x 64 B: records of this vertex and the next two (TMA)
constexpr int kOffBar = kOffRec + 192;    // mma bar, TMA bar, 3 record bars
constexpr int kOffTmem = kOffBar + 40;
constexpr int kOffFlag = kOffTmem + 4;
constexpr int kSmemUsed = kOffFlag + 4;
constexpr int kSmemBytes = kSmemUsed + 1024;  // room to align the base
constexpr uint32_t kTmemCols = 128;

constexpr uint32_t kIdescG1 = tc::idesc_bf16(128, 64, 0, 0);
constexpr uint32_t kIdescG1mn = tc::idesc_bf16(128, 64, 1, 0);
constexpr uint32_t kIdescG2 = tc::idesc_bf16(64, 64, 0, 0);
constexpr uint32_t kIdescG2mn = tc::idesc_bf16(64, 64, 0, 1);

// 32 lanes x 32 bits, 32 consecutive columns per thread; the values are valid
// after tmem_wait_ld (several loads may be in flight before one wait).
__device__ __forceinline__ void tmem_ld_x32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// 16 lanes x 32 bits in two halves: threads 0-15 read lanes 0-15 of the
// warp's quadrant at columns [c, c + 32), threads 16-31 the same lanes at
// columns [c + 32, c + 64) -- the rows of an M = 64 result, all 32 threads busy.
__device__ __forceinline__ void tmem_ld_16x32bx2_x32(uint32_t taddr, uint32_t (&r)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.16x32bx2.x32.b32 "
      "{%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32], 32;"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr)
      : "memory");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&p);
}

// 32 FP32 values -> 16-byte chunks [c0, c0+4) of one 128-byte BF16 row of a
// 128B-swizzled tile (chunk j lands at j ^ (row % 8)).
__device__ __forceinline__ void store_half_row(unsigned char* tile, int row, int c0, const uint32_t (&v)[32]) {
  uint4* base = reinterpret_cast<uint4*>(tile + row * 128);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint4 q;
    q.x = pack_bf16(__uint_as_float(v[8 * j + 0]), __uint_as_float(v[8 * j + 1]));
    q.y = pack_bf16(__uint_as_float(v[8 * j + 2]), __uint_as_float(v[8 * j + 3]));
    q.z = pack_bf16(__uint_as_float(v[8 * j + 4]), __uint_as_float(v[8 * j + 5]));
    q.w = pack_bf16(__uint_as_float(v[8 * j + 6]), __uint_as_float(v[8 * j + 7]));
    base[(c0 + j) ^ (row & 7)] = q;
  }
}

// Entry e (b = e % 8, a = e / 8) of the 8 x 8 padded image of a compact
// chi x chi message; chi = 0 marks a padding leg, whose message is 1 at (0, 0).
__device__ __forceinline__ float padded_msg(const float* m, int off, int chi, int e) {
  const int b = e & 7, a = e >> 3;
  if (chi == 0) return e == 0 ? 1.f : 0.f;
  return (b < chi && a < chi) ? m[off + b + chi * a] : 0.f;
}

__device__ __forceinline__ int rec_chi(int chi4, int p) { return (chi4 >> (8 * p)) & 0xff; }

// Normalise one 8 x 8 message held by a warp (two values per lane), store its
// compact chi x chi part as FP32, and (want_diff) return
// message_diff(new, old) = 1 - <a, b>^2 / (|a|^2 |b|^2)
// (abstractbeliefpropagationcache.jl:32-36) against the previous message's
// entries o0, o1 (same positions, zero outside chi x chi).  It is formed in
// FP32 as s - s^2 / 4 with s = |a/|a| - b/|b||^2 (= 2 - 2 cos, so
// s - s^2 / 4 = 1 - cos^2 for either sign of cos): no cancellation, so the
// diff keeps FP32's relative accuracy however small it is, and the FP64 pipe,
// which three FP64 warp reductions per message kept as busy as the whole
// contraction, is not used.  Entries outside chi x chi are exact zeros.
__device__ __forceinline__ double tc_finalize(const float* res, float o0, float o1, float* out, int chi, int normalize,
                                              bool want_diff, int lane) {
  const float x0 = res[lane], x1 = res[lane + 32];
  float ss = fmaf(x0, x0, x1 * x1);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ss += __shfl_xor_sync(0xffffffffu, ss, o);
  const float sc = (normalize && ss > 0.f) ? rsqrtf(ss) : 1.f;
  const float n0 = x0 * sc, n1 = x1 * sc;
  const int b = lane & 7, a0 = lane >> 3, a1 = a0 + 4;
  const bool v0 = b < chi && a0 < chi, v1 = b < chi && a1 < chi;
  const int i0 = b + chi * a0, i1 = b + chi * a1;
  if (v0) out[i0] = n0;
  if (v1) out[i1] = n1;
  double diff = 0.0;
  if (want_diff) {
    float na = fmaf(n0, n0, n1 * n1), nb = fmaf(o0, o0, o1 * o1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      na += __shfl_xor_sync(0xffffffffu, na, o);
      nb += __shfl_xor_sync(0xffffffffu, nb, o);
    }
    const float ia = rsqrtf(na), ib = rsqrtf(nb);
    const float d0 = fmaf(n0, ia, -o0 * ib), d1 = fmaf(n1, ia, -o1 * ib);
    float sd = fmaf(d0, d0, d1 * d1);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sd += __shfl_xor_sync(0xffffffffu, sd, o);
    diff = (double)fmaf(-0.25f * sd, sd, sd);
  }
  return diff;
}
}  // namespace

namespace {

// Outgoing messages of one leg pair (x, y) from its environment
// G[(ax,ay),(bx,by)] (ket row ax + 8 ay, bra column bx + 8 by; M = 64 layout:
// warp w holds rows 16 w .. 16 w + 15 in lanes 0-15 of its TMEM quadrant).
// Lane l works on row r = l % 16 (ax = r % 8, ay = 2 w + r / 8) and the column
// half h = l / 16 (by = 4 h .. 4 h + 3):
//   out_y[by, ay] = sum_{ax,bx} G Mx[bx, ax]  -> res_y (complete within the warp)
//   out_x[bx, ax] = sum_{ay,by} G My[by, ay]  -> per-warp partials part[warp][ax][bx]
__device__ __forceinline__ void pair_epilogue(uint32_t taddr, const float* Mx, const float* My, float* res_y,
                                              float* part, int warp, int lane) {
  const int r = lane & 15, h = lane >> 4;
  const int ax = r & 7, ay = 2 * warp + (r >> 3);
  float2 mx2[4], p2[4], q2[4];  // pairs (bx, bx + 1); q2 holds the even / odd bx halves of q
  float my[4], q[4], p[8];
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    mx2[k] = *reinterpret_cast<const float2*>(Mx + 2 * k + 8 * ax);  // Mx[bx = 2k, 2k + 1; ax]
    p2[k] = make_float2(0.f, 0.f);
    q2[k] = make_float2(0.f, 0.f);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) my[i] = My[4 * h + i + 8 * ay];  // My[by = 4 h + i, ay]
  uint32_t g[32];
  tmem_ld_16x32bx2_x32(taddr, g);
  tmem_wait_ld();
#pragma unroll
  for (int jj = 0; jj < 32; jj += 2) {
    const int k = (jj & 7) >> 1, i = jj >> 3;  // columns 32 h + jj, + 1: bx = 2k, 2k + 1; by = 4 h + i
    const float2 gv = make_float2(__uint_as_float(g[jj]), __uint_as_float(g[jj + 1]));
    q2[i] = __ffma2_rn(gv, mx2[k], q2[i]);
    p2[k] = __ffma2_rn(gv, make_float2(my[i], my[i]), p2[k]);
  }
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    q[i] = q2[i].x + q2[i].y;
    p[2 * i] = p2[i].x;
    p[2 * i + 1] = p2[i].y;
  }
  // q: sum over ax (lane bits 0-2), scattered: lanes ax, ax ^ 1 end with by = 4 h + 2 ax2 + ax1
  {
    const bool up = ax & 4;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const float send = up ? q[i] : q[i + 2];
      const float keep = up ? q[i + 2] : q[i];
      q[i] = keep + __shfl_xor_sync(0xffffffffu, send, 4);
    }
  }
  {
    const bool up = ax & 2;
    const float send = up ? q[0] : q[1];
    const float keep = up ? q[1] : q[0];
    q[0] = keep + __shfl_xor_sync(0xffffffffu, send, 2);
  }
  q[0] += __shfl_xor_sync(0xffffffffu, q[0], 1);
  if ((ax & 1) == 0) {
    const int by = 4 * h + 2 * ((ax >> 2) & 1) + ((ax >> 1) & 1);
    res_y[by + 8 * ay] = q[0];
  }
  // p: sum over the column half (lane bit 4) and the warp's two ay (lane bit 3), scattered
  {
    const bool up = lane & 16;
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      const float send = up ? p[i] : p[i + 4];
      const float keep = up ? p[i + 4] : p[i];
      p[i] = keep + __shfl_xor_sync(0xffffffffu, send, 16);
    }
  }
  {
    const bool up = lane & 8;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
      const float send = up ? p[i] : p[i + 2];
      const float keep = up ? p[i + 2] : p[i];
      p[i] = keep + __shfl_xor_sync(0xffffffffu, send, 8);
    }
  }
  {
    const int bx0 = 4 * ((lane >> 4) & 1) + 2 * ((lane >> 3) & 1);
    part[warp * 64 + ax * 8 + bx0] = p[0];
    part[warp * 64 + ax * 8 + bx0 + 1] = p[1];
  }
}

}  // namespace

// One CTA walks recs[blockIdx.x], recs[blockIdx.x + gridDim.x], ... (one
// record per vertex of the work list, in list order; Z at zimg + slot * 8192).
// The records arrive by 64-byte bulk copies two vertices ahead into a ring
// of three, so no thread reads a record from global memory: a load still in
// flight would hold up the next CTA barrier.
// err (device) receives GBTN_ERR_TIMEOUT when a bounded wait gives up; the CTA
// then drains its own copy and MMAs in flight, frees its TMEM and returns.
__global__ void __launch_bounds__(kTcThreads, kTcBlocksPerSm)
    tc_vertex_kernel(const TcRec* __restrict__ recs, int nwork, const __nv_bfloat16* __restrict__ zimg,
                     const float* msg_in,
                     float* msg_out, double* diffs, const int* converged, int normalize, int want_diff, int* err,
                     unsigned int extra_tx) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* Z = sm + kOffZ;
  unsigned char* KT = sm + kOffKT;  // K12 | K34, later the two T12 tiles
  unsigned char* T34 = sm + kOffT34;
  float* PART = reinterpret_cast<float*>(sm + kOffPart);
  float* MSG = reinterpret_cast<float*>(sm + kOffMsg);
  float* RES = reinterpret_cast<float*>(sm + kOffRes);
  const TcRec* REC = reinterpret_cast<const TcRec*>(sm + kOffRec);
  uint64_t* mma_bar = reinterpret_cast<uint64_t*>(sm + kOffBar);
  uint64_t* tma_bar = mma_bar + 1;
  uint64_t* rec_bar = mma_bar + 2;  // [3]
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kOffTmem);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(sm + kOffFlag);

  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(mma_bar, 2);  // one commit from each MMA issuer
    tc::mbar_init(tma_bar, 1);
    for (int k = 0; k < 3; ++k) tc::mbar_init(rec_bar + k, 1);
    tc::fence_mbar_init();
    *abort_flag = 0;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's TMEM lanes
  // operand descriptors at offset 0 (K-major tiles: LBO 16 B, SBO 1024 B; Z read
  // MN-major: LBO 8192 B between the two site halves), formed by the issuing thread
  auto descs = [&](uint64_t& dZk, uint64_t& dZmn, uint64_t& dKT, uint64_t& dT34) {
    dZk = tc::smem_desc(tc::smem_u32(Z), 16, 1024);
    dZmn = tc::smem_desc(tc::smem_u32(Z), 8192, 1024);
    dKT = tc::smem_desc(tc::smem_u32(KT), 16, 1024);
    dT34 = tc::smem_desc(tc::smem_u32(T34), 16, 1024);
  };

  // thread-0 bookkeeping of the asynchronous work in flight
  uint32_t mma_phase = 0, tma_phase = 0;
  int tma_pending = 0, mma_pending = 0;
  auto issue_z = [&](int slot) {
    tc::mbar_expect_tx(tma_bar, kZBytes + extra_tx);
    tc::tma_load_1d(Z, zimg + (size_t)slot * kZElems, kZBytes, tma_bar);
    tma_pending = 1;
  };
  auto wait_z = [&]() -> bool {
    const bool ok = tc::mbar_wait(tma_bar, tma_phase, kWaitNs);
    if (ok) {
      tma_phase ^= 1;
      tma_pending = 0;
    }
    return ok;
  };
  auto wait_mma = [&]() -> bool {
    const bool ok = tc::mbar_wait(mma_bar, mma_phase, kWaitNs);
    if (ok) {
      mma_phase ^= 1;
      mma_pending = 0;
    }
    return ok;
  };
  // record i of this CTA's walk goes to ring entry i % 3 (use i / 3)
  int rec_pending[3] = {0, 0, 0};
  uint32_t rec_par[3] = {0, 0, 0};
  auto issue_rec = [&](int i, int wv) {
    const int k = i % 3;
    tc::mbar_expect_tx(rec_bar + k, (uint32_t)sizeof(TcRec));
    tc::tma_load_1d(sm + kOffRec + k * sizeof(TcRec), recs + wv, (uint32_t)sizeof(TcRec), rec_bar + k);
    rec_pending[k] = 1;
    rec_par[k] = (uint32_t)(i / 3) & 1;
  };
  auto wait_rec = [&](int i) -> bool {
    const int k = i % 3;
    const bool ok = tc::mbar_wait(rec_bar + k, rec_par[k], kWaitNs);
    if (ok) rec_pending[k] = 0;
    return ok;
  };

  const int q0 = t, q1 = t + 128;  // this thread's entries of the 4 x 64 message block
  const int e = t & 63;
  const int G = gridDim.x;
  int w = blockIdx.x;
  float cm0 = 0.f, cm1 = 0.f;  // current vertex's incoming-message entries q0, q1
  int cnet = 0;
  if (t == 0 && w < nwork) {
    issue_rec(0, w);
    if (w + G < nwork) issue_rec(1, w + G);
    const bool ok = wait_rec(0);
    *abort_flag = ok ? 0 : 1;
    if (ok) issue_z(REC[0].slot);
  }
  __syncthreads();
  const bool started = !*abort_flag;  // read by every thread after the barrier: uniform
  if (w < nwork && started) {
    const TcRec& r = REC[0];
    cnet = r.net;
    const int c4 = r.chi4;
    cm0 = padded_msg(msg_in, r.in_off[q0 >> 6], rec_chi(c4, q0 >> 6), e);
    cm1 = padded_msg(msg_in, r.in_off[q1 >> 6], rec_chi(c4, q1 >> 6), e);
  }
  // a wait that gives up inside the loop is seen by every thread after the next barrier
  for (int it = 0; started && w < nwork; w += G, ++it) {
    const TcRec& cr = REC[it % 3];  // this vertex (complete since the previous iteration)
    const TcRec& nr = REC[(it + 1) % 3];
    const int wn = w + G;
    // the next vertex's record must be here before the barrier below makes it visible
    if (t == 0 && wn < nwork && !wait_rec(it + 1)) *abort_flag = 1;
    const int out_off_w = cr.out_off[warp];
    const int out_de_w = cr.out_de[warp];
    const int cchi4 = cr.chi4;
    const int chi_w = rec_chi(cchi4, warp);
    // the previous outgoing message of this warp's leg (message_diff), loaded now, used last
    float old0 = 0.f, old1 = 0.f;
    if (want_diff) {
      const int b = lane & 7, a0 = lane >> 3;
      if (b < chi_w && a0 < chi_w) old0 = msg_in[out_off_w + b + chi_w * a0];
      if (b < chi_w && a0 + 4 < chi_w) old1 = msg_in[out_off_w + b + chi_w * (a0 + 4)];
    }
    float nm0 = 0.f, nm1 = 0.f;

    if (converged && converged[cnet]) {  // network done: carry its messages forward
      const int p0 = q0 >> 6, p1 = q1 >> 6;
      const int c0 = rec_chi(cchi4, p0), c1 = rec_chi(cchi4, p1);
      if (e < c0 * c0) msg_out[cr.out_off[p0] + e] = msg_in[cr.out_off[p0] + e];
      if (e < c1 * c1) msg_out[cr.out_off[p1] + e] = msg_in[cr.out_off[p1] + e];
      if (t == 0 && !*abort_flag) {
        const bool ok = wait_z();
        *abort_flag = ok ? 0 : 1;
        if (ok && wn < nwork) issue_z(nr.slot);
      }
      __syncthreads();
      if (*abort_flag) break;
      // every thread is past the previous vertex: its ring entry takes the one after next
      if (t == 0 && wn + G < nwork) issue_rec(it + 2, wn + G);
      if (wn < nwork) {
        cm0 = padded_msg(msg_in, nr.in_off[q0 >> 6], rec_chi(nr.chi4, q0 >> 6), e);
        cm1 = padded_msg(msg_in, nr.in_off[q1 >> 6], rec_chi(nr.chi4, q1 >> 6), e);
        cnet = nr.net;
      }
      continue;
    }

    MSG[q0] = cm0;
    MSG[q1] = cm1;
    __syncthreads();
    if (*abort_flag) break;
    // every thread is past the previous vertex: its ring entry takes the one after next
    if (t == 0 && wn + G < nwork) issue_rec(it + 2, wn + G);
    int nsl = -1, nin0 = 0, nin1 = 0, nnet = 0, nchi0 = 8, nchi1 = 8;
    if (wn < nwork) {
      nsl = nr.slot;
      nin0 = nr.in_off[q0 >> 6];
      nin1 = nr.in_off[q1 >> 6];
      nnet = nr.net;
      const int n4 = nr.chi4;
      nchi0 = rec_chi(n4, q0 >> 6);
      nchi1 = rec_chi(n4, q1 >> 6);
    }
    {
      // Kronecker products: threads 0-63 build K12 = M1 (x) M2, 64-127 K34 = M3 (x) M4;
      // row n = b_a + 8 b_b, column k = a_a + 8 a_b (16-byte chunk a_b), value M_a[b_a,a_a] M_b[b_b,a_b]
      const int n = t & 63, ba = n & 7, bb = n >> 3;
      const float* Ma = MSG + (t < 64 ? 0 : 128);
      const float* Mb = Ma + 64;
      float2 ma[4];
#pragma unroll
      for (int k = 0; k < 4; ++k) ma[k] = make_float2(Ma[ba + 16 * k], Ma[ba + 16 * k + 8]);
      uint4* row = reinterpret_cast<uint4*>(KT + (t < 64 ? 0 : 8192) + n * 128);
#pragma unroll
      for (int ab = 0; ab < 8; ++ab) {
        const float mb = Mb[bb + 8 * ab];
        const float2 mb2 = make_float2(mb, mb);
        uint32_t w[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const float2 pr = __fmul2_rn(ma[k], mb2);
          w[k] = pack_bf16(pr.x, pr.y);
        }
        row[ab ^ (n & 7)] = make_uint4(w[0], w[1], w[2], w[3]);
      }
      tc::fence_proxy_async_smem();
    }
    if (t == 0) *abort_flag = wait_z() ? 0 : 1;
    __syncthreads();
    if (*abort_flag) break;

    // ---- GEMM1 -> columns [0,64), GEMM1' -> [64,128) (M = 128) ----
    // descriptors: per-CTA bases (dZk, dZmn, dKT, dT34) plus the operand's
    // byte offset in 16-byte units (the start-address field of the descriptor)
    // Two issuers: thread 0 the GEMM1 chain, thread 32 the GEMM1' chain (separate
    // accumulators).  A thread waits ~70 cycles per small MMA it issues; two
    // issuers overlap in the tensor pipe.
    if (t == 0 || t == 32) {
      tc::tc_fence_after();
      uint64_t dZk, dZmn, dKT, dT34;
      descs(dZk, dZmn, dKT, dT34);
      if (t == 0) {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          tc::mma_bf16(tmem + 0, dZk + ((32 * kk) >> 4), dKT + ((32 * kk) >> 4), kIdescG1, kk > 0);
      } else {
#pragma unroll
        for (int kk = 0; kk < 4; ++kk)
          tc::mma_bf16(tmem + 64, dZmn + ((2048 * kk) >> 4), dKT + ((8192 + 32 * kk) >> 4), kIdescG1mn, kk > 0);
      }
      tc::mma_commit(mma_bar);
    }
    if (t == 0) {
      mma_pending = 1;
      *abort_flag = wait_mma() ? 0 : 1;
    }
    __syncthreads();
    if (*abort_flag) break;
    tc::tc_fence_after();
    {
      // row t = (s, c) of D1 / D1' -> row c of tile s of T12 / T34 (K = (s, c') = 128)
      const int s = t >> 6, c = t & 63;
      uint32_t d[2][32];
      tmem_ld_x32(trow + 0, d[0]);
      tmem_ld_x32(trow + 32, d[1]);
      tmem_wait_ld();
      store_half_row(KT + 8192 * s, c, 0, d[0]);  // T12 overwrites the Kronecker products (their MMAs are done)
      store_half_row(KT + 8192 * s, c, 4, d[1]);
      tmem_ld_x32(trow + 64, d[0]);
      tmem_ld_x32(trow + 96, d[1]);
      tmem_wait_ld();
      store_half_row(T34 + 8192 * s, c, 0, d[0]);
      store_half_row(T34 + 8192 * s, c, 4, d[1]);
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    // ---- GEMM2 -> G34 in columns [0,64), GEMM2' -> G12 in [64,128) (M = 64, K = 128) ----
    if (t == 0 || t == 32) {
      tc::tc_fence_after();
      uint64_t dZk, dZmn, dKT, dT34;
      descs(dZk, dZmn, dKT, dT34);
      if (t == 0) {
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          const uint32_t o = (8192 * (kk >> 2) + 32 * (kk & 3)) >> 4;
          tc::mma_bf16(tmem + 0, dKT + o, dZk + o, kIdescG2, kk > 0);
        }
      } else {
#pragma unroll
        for (int kk = 0; kk < 8; ++kk) {
          const uint32_t o = (8192 * (kk >> 2) + 32 * (kk & 3)) >> 4;
          tc::mma_bf16(tmem + 64, dT34 + o, dZmn + ((2048 * kk) >> 4), kIdescG2mn, kk > 0);
        }
      }
      tc::mma_commit(mma_bar);
    }
    if (t == 0) mma_pending = 1;
    // the next vertex's incoming messages, ahead of use
    if (nsl >= 0) {
      nm0 = padded_msg(msg_in, nin0, nchi0, e);
      nm1 = padded_msg(msg_in, nin1, nchi1, e);
    }
    if (t == 0) {
      const bool ok = wait_mma();
      *abort_flag = ok ? 0 : 1;
      if (ok && nsl >= 0) issue_z(nsl);  // Z is free: fetch the next vertex's image
    }
    __syncthreads();
    if (*abort_flag) break;
    tc::tc_fence_after();
    // legs (3,4): out4 complete per warp, out3 as partials; legs (1,2): out2, out1 partials
    pair_epilogue(trow + 0, MSG + 128, MSG + 192, RES + 192, PART, warp, lane);
    pair_epilogue(trow + 64, MSG, MSG + 64, RES + 64, PART + 256, warp, lane);
    tc::tc_fence_before();
    __syncthreads();
    {
      const float* pp = PART + (t < 64 ? 0 : 256);
      const int u = t & 63;
      RES[(t < 64 ? 128 : 0) + u] = pp[u] + pp[64 + u] + pp[128 + u] + pp[192 + u];  // out3 | out1
    }
    __syncthreads();
    if (chi_w > 0) {  // warp-uniform: a padding leg has no outgoing message
      const double df = tc_finalize(RES + 64 * warp, old0, old1, msg_out + out_off_w, chi_w, normalize,
                                    want_diff != 0, lane);
      if (want_diff && lane == 0) diffs[out_de_w] = df;
    }
    cm0 = nm0;
    cm1 = nm1;
    cnet = nnet;
  }

  // drain: after a timeout, wait (bounded) for this CTA's own copies and MMAs;
  // record copies issued for vertices the walk did not reach land before exit
  if (t == 0) {
    if (*abort_flag) {
      atomicExch(err, (int)GBTN_ERR_TIMEOUT);
      if (tma_pending) wait_z();
      if (mma_pending) wait_mma();
    }
    for (int k = 0; k < 3; ++k)
      if (rec_pending[k]) tc::mbar_wait(rec_bar + k, rec_par[k], kWaitNs);
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

namespace {

// Swizzled BF16 image of Z for every slot: image element (s, c1, c2) with
// c1 = l1 + 8 l2, c2 = l3 + 8 l4 goes to row r = 64 s + c2, 16-byte chunk
// (c1 / 8) ^ (r % 8); it holds A[s, l1..lk] when every l_p is inside the
// vertex's bond dimension (l_p = 0 on a padding leg p >= k) and zero otherwise.
__global__ void build_zimg_kernel(const int* __restrict__ slot_vertex, int nslot, const VDesc* __restrict__ vd,
                                  const double* __restrict__ fac, __nv_bfloat16* __restrict__ zimg) {
  const int slot = blockIdx.x;
  if (slot >= nslot) return;
  const VDesc d = vd[slot_vertex[slot]];
  const double* a = fac + d.a_off;
  __nv_bfloat16* z = zimg + (size_t)slot * kZElems;
  for (int idx = threadIdx.x; idx < (int)kZElems; idx += blockDim.x) {
    const int s = idx & 1, c1 = (idx >> 1) & 63, c2 = idx >> 7;
    const int l[4] = {c1 & 7, c1 >> 3, c2 & 7, c2 >> 3};
    bool in = true;
    long long src = s;
#pragma unroll
    for (int p = 0; p < 4; ++p) {
      if (p < d.k) {
        in = in && l[p] < d.chi[p];
        src += (long long)l[p] * d.st[p];
      } else {
        in = in && l[p] == 0;
      }
    }
    const int r = 64 * s + c2;
    z[r * 64 + (((c1 >> 3) ^ (r & 7)) << 3) + (c1 & 7)] = __double2bfloat16(in ? a[src] : 0.0);
  }
}

}  // namespace

bool tc_native(const VDesc& d) {
  if (d.k != 4 || d.d != 2) return false;
  for (int p = 0; p < 4; ++p)
    if (d.chi[p] != 8) return false;
  return true;
}

bool tc_paddable(const VDesc& d) {
  if (d.k < 1 || d.k > 4 || d.d != 2) return false;
  for (int p = 0; p < d.k; ++p)
    if (d.chi[p] < 1 || d.chi[p] > 8) return false;
  return true;
}

TcRec tc_record(const VDesc& d, const std::vector<long long>& msg_off) {
  TcRec r{};
  r.chi4 = 0;
  for (int p = 0; p < 4; ++p) {
    if (p < d.k) {
      r.in_off[p] = (int)msg_off[d.in_de[p]];
      r.out_off[p] = (int)msg_off[d.out_de[p]];
      r.out_de[p] = d.out_de[p];
      r.chi4 |= d.chi[p] << (8 * p);
    } else {
      r.in_off[p] = 0;
      r.out_off[p] = 0;
      r.out_de[p] = -1;
    }
  }
  r.net = d.net;
  r.slot = -1;
  return r;
}

void launch_build_zimg(const int* slot_vertex, int nslot, const VDesc* vd, const double* fac, __nv_bfloat16* zimg,
                       cudaStream_t s) {
  if (nslot == 0) return;
  build_zimg_kernel<<<nslot, 256, 0, s>>>(slot_vertex, nslot, vd, fac, zimg);
  GBTN_CUDA(cudaGetLastError());
}

void tc_set_test_extra_tx(unsigned int bytes) { g_tc_test_extra_tx = bytes; }

void launch_tc_vertices(const TcRec* recs, int nwork, const __nv_bfloat16* zimg,
                        const float* msg_in, float* msg_out, double* diffs, const int* converged, int normalize,
                        int want_diff, int* err, cudaStream_t s) {
  if (nwork == 0) return;
  static int nsm = 0;
  if (nsm == 0) {
    int dev = 0;
    GBTN_CUDA(cudaGetDevice(&dev));
    GBTN_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
  }
  GBTN_CUDA(cudaFuncSetAttribute(tc_vertex_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kSmemBytes));
  const int slots = kTcBlocksPerSm * nsm;
  const int grid = nwork < slots ? nwork : slots;
  tc_vertex_kernel<<<grid, kTcThreads, kSmemBytes, s>>>(recs, nwork, zimg, msg_in, msg_out, diffs,
                                                         converged, normalize, want_diff, err, g_tc_test_extra_tx);
  GBTN_CUDA(cudaGetLastError());
}

}  // namespace gbtn
