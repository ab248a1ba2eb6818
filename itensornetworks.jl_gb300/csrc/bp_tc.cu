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
// are 64 x 64 x 64 FP32 contractions on the CUDA cores.  Each output is
// normalised with an FP64 sum of squares and written as an FP32 message
// (updated_message, src/caches/abstractbeliefpropagationcache.jl:225-239).
//
// Per vertex: one 16 KB TMA bulk copy of the pre-swizzled BF16 image of Z,
// 16 tcgen05.mma instructions accumulating in FP32 in TMEM (128 columns,
// reused by the three MMA phases), 128 threads.  Four CTAs share an SM
// (52 KB of shared memory each: the Kronecker products, then T12, then the
// environment G reuse one region), so one CTA's MMAs overlap the others'
// epilogues; each CTA also overlaps GEMM2' with the G34 epilogue, copies the
// next vertex's Z while finishing the current one, and loads the next
// vertex's messages into registers ahead of time.
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

// shared-memory carve-up (bytes from a 1024-aligned base)
constexpr int kOffZ = 0;           // 16 KB: Z image (TMA destination)
constexpr int kOffKT = 16384;      // K12 | K34 (2 x 8 KB), then T12 (16 KB), then G (16.25 KB)
constexpr int kGStride = 65;       // padded FP32 row of the 64 x 64 environment
constexpr int kKTBytes = 17408;    // >= 64 * 65 * 4, multiple of 1024
constexpr int kOffT34 = kOffKT + kKTBytes;
constexpr int kOffMsg = kOffT34 + 16384;  // 4 x 64 FP32 incoming messages
constexpr int kOffRes = kOffMsg + 1024;   // 4 x 64 FP32 outgoing messages
constexpr int kOffBar = kOffRes + 1024;   // mma bar, TMA bar
constexpr int kOffTmem = kOffBar + 16;
constexpr int kOffFlag = kOffTmem + 4;
constexpr int kSmemUsed = kOffFlag + 4;
constexpr int kSmemBytes = kSmemUsed + 1024;  // room to align the base
constexpr uint32_t kTmemCols = 128;

static_assert(kOffT34 % 1024 == 0, "swizzled tiles need 1024-byte alignment");
static_assert(64 * kGStride * 4 <= kKTBytes, "environment does not fit its region");

constexpr uint32_t kIdescG1 = tc::idesc_bf16(128, 64, 0, 0);
constexpr uint32_t kIdescG1mn = tc::idesc_bf16(128, 64, 1, 0);
constexpr uint32_t kIdescG2 = tc::idesc_bf16(128, 128, 0, 0);
constexpr uint32_t kIdescG2mn = tc::idesc_bf16(128, 128, 0, 1);

__device__ __forceinline__ double tc_warp_sum(double x) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// 32 lanes x 32 bits, 32 consecutive columns per thread.
__device__ __forceinline__ void tmem_ld_x32(uint32_t taddr, float (&v)[32]) {
  uint32_t r[32];
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
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 p = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&p);
}

// 32 FP32 values -> 16-byte chunks [c0, c0+4) of one 128-byte BF16 row of a
// 128B-swizzled tile (chunk j lands at j ^ (row % 8)).
__device__ __forceinline__ void store_half_row(unsigned char* tile, int row, int c0, const float (&v)[32]) {
  uint4* base = reinterpret_cast<uint4*>(tile + row * 128);
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    uint4 q;
    q.x = pack_bf16(v[8 * j + 0], v[8 * j + 1]);
    q.y = pack_bf16(v[8 * j + 2], v[8 * j + 3]);
    q.z = pack_bf16(v[8 * j + 4], v[8 * j + 5]);
    q.w = pack_bf16(v[8 * j + 6], v[8 * j + 7]);
    base[(c0 + j) ^ (row & 7)] = q;
  }
}

// Normalise one 8 x 8 message held by a warp (two values per lane) with an
// FP64 sum of squares, store it as FP32, and (want_diff) return
// message_diff(new, old) (abstractbeliefpropagationcache.jl:32-36).
__device__ __forceinline__ double tc_finalize(const float* res, const float* old, float* out, int normalize,
                                              bool want_diff, int lane) {
  const float x0 = res[lane], x1 = res[lane + 32];
  const double ss = tc_warp_sum((double)x0 * (double)x0 + (double)x1 * (double)x1);
  const float sc = (normalize && ss > 0.0) ? (float)rsqrt(ss) : 1.f;
  const float n0 = x0 * sc, n1 = x1 * sc;
  float o0 = 0.f, o1 = 0.f;
  if (want_diff) {
    o0 = old[lane];
    o1 = old[lane + 32];
  }
  __syncwarp();
  out[lane] = n0;
  out[lane + 32] = n1;
  double diff = 0.0;
  if (want_diff) {
    const double a0 = n0, a1 = n1, b0 = o0, b1 = o1;
    const double dot = tc_warp_sum(a0 * b0 + a1 * b1);
    const double na = tc_warp_sum(a0 * a0 + a1 * a1);
    const double nb = tc_warp_sum(b0 * b0 + b1 * b1);
    diff = 1.0 - (dot * dot) / (na * nb);
  }
  return diff;
}

}  // namespace

namespace {

// D2 / D2' diagonal block of this thread's row (s = row / 64) summed over s
// into G[c][.] (c = row % 64): rows with s = 0 store, rows with s = 1 add.
__device__ __forceinline__ void diag_to_env(uint32_t taddr, float* G, int t) {
  const int s = t >> 6, c = t & 63;
  float d0[32], d1[32];
  tmem_ld_x32(taddr + 64 * s, d0);
  tmem_ld_x32(taddr + 64 * s + 32, d1);
  float* g = G + c * kGStride;
  if (s == 0) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      g[j] = d0[j];
      g[32 + j] = d1[j];
    }
  }
  __syncthreads();
  if (s == 1) {
#pragma unroll
    for (int j = 0; j < 32; ++j) {
      g[j] += d0[j];
      g[32 + j] += d1[j];
    }
  }
  __syncthreads();
}

// Outgoing messages of one leg pair from its environment G[(ax,ay),(bx,by)]:
// threads 0-63 contract the second leg with Mx (result on the first leg),
// threads 64-127 contract the first leg with My (result on the second leg).
__device__ __forceinline__ void env_to_out(const float* G, const float* Mx, const float* My, float* res_first,
                                           float* res_second, int t) {
  const int u = t & 63, bx = u & 7, ax = u >> 3;
  float acc = 0.f;
  if (t < 64) {
#pragma unroll
    for (int ay = 0; ay < 8; ++ay)
#pragma unroll
      for (int by = 0; by < 8; ++by) acc = fmaf(G[(ax + 8 * ay) * kGStride + bx + 8 * by], Mx[by + 8 * ay], acc);
    res_first[u] = acc;
  } else {
#pragma unroll
    for (int ay = 0; ay < 8; ++ay)
#pragma unroll
      for (int by = 0; by < 8; ++by) acc = fmaf(G[(ay + 8 * ax) * kGStride + by + 8 * bx], My[by + 8 * ay], acc);
    res_second[u] = acc;
  }
}

}  // namespace

// One CTA walks work[blockIdx.x], work[blockIdx.x + gridDim.x], ...; vertex v
// uses image slot vslot[v] (Z at zimg + slot * 8192, offsets in recs[slot]).
// err (device) receives GBTN_ERR_TIMEOUT when a bounded wait gives up; the CTA
// then drains its own copies and MMAs in flight, frees its TMEM and returns.
__global__ void __launch_bounds__(kTcThreads, kTcBlocksPerSm)
    tc_vertex_kernel(const int* __restrict__ work, int nwork, const int* __restrict__ vslot,
                     const TcRec* __restrict__ recs, const __nv_bfloat16* __restrict__ zimg, const float* msg_in,
                     float* msg_out, double* diffs, const int* converged, int normalize, int want_diff, int* err) {
  extern __shared__ unsigned char smem_raw[];
  unsigned char* sm = reinterpret_cast<unsigned char*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
  unsigned char* Z = sm + kOffZ;
  unsigned char* KT = sm + kOffKT;  // K12 | K34, later T12, later G
  unsigned char* T34 = sm + kOffT34;
  float* G = reinterpret_cast<float*>(KT);
  float* MSG = reinterpret_cast<float*>(sm + kOffMsg);
  float* RES = reinterpret_cast<float*>(sm + kOffRes);
  uint64_t* mma_bar = reinterpret_cast<uint64_t*>(sm + kOffBar);
  uint64_t* tma_bar = mma_bar + 1;
  uint32_t* tmem_slot = reinterpret_cast<uint32_t*>(sm + kOffTmem);
  volatile int* abort_flag = reinterpret_cast<volatile int*>(sm + kOffFlag);

  const int t = threadIdx.x, warp = t >> 5, lane = t & 31;
  if (warp == 0) {
    tc::tmem_alloc(tmem_slot, kTmemCols);
    tc::tmem_relinquish();
  }
  if (t == 0) {
    tc::mbar_init(mma_bar, 1);
    tc::mbar_init(tma_bar, 1);
    tc::fence_mbar_init();
    *abort_flag = 0;
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  const uint32_t tmem = *tmem_slot;
  const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's TMEM lanes

  // thread-0 bookkeeping of the asynchronous work in flight
  uint32_t mma_phase = 0, tma_phase = 0;
  int tma_pending = 0, mma_pending = 0;
  auto issue_z = [&](int slot) {
    tc::mbar_expect_tx(tma_bar, kZBytes);
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
  auto commit = [&]() {
    tc::mma_commit(mma_bar);
    mma_pending = 1;
  };

  const int q0 = t, q1 = t + 128;  // this thread's entries of the 4 x 64 message block
  const int e = t & 63;
  int w = blockIdx.x;
  float cm0 = 0.f, cm1 = 0.f;  // current vertex's incoming-message entries q0, q1
  int cnet = 0;
  if (w < nwork) {
    const int sl = vslot[work[w]];
    if (t == 0) issue_z(sl);
    cnet = recs[sl].net;
    cm0 = msg_in[recs[sl].in_off[q0 >> 6] + e];
    cm1 = msg_in[recs[sl].in_off[q1 >> 6] + e];
  }
  for (; w < nwork; w += gridDim.x) {
    const int sl = vslot[work[w]];
    const int out_off_w = recs[sl].out_off[warp];
    const int out_de_w = recs[sl].out_de[warp];
    // next vertex: record now, messages later in this iteration
    const int wn = w + gridDim.x;
    int nsl = -1, nin0 = 0, nin1 = 0, nnet = 0;
    if (wn < nwork) {
      nsl = vslot[work[wn]];
      nin0 = recs[nsl].in_off[q0 >> 6];
      nin1 = recs[nsl].in_off[q1 >> 6];
      nnet = recs[nsl].net;
    }
    float nm0 = 0.f, nm1 = 0.f;

    if (converged && converged[cnet]) {  // network done: carry its messages forward
      const int o0 = recs[sl].out_off[q0 >> 6], o1 = recs[sl].out_off[q1 >> 6];
      msg_out[o0 + e] = msg_in[o0 + e];
      msg_out[o1 + e] = msg_in[o1 + e];
      if (t == 0) {
        const bool ok = wait_z();
        *abort_flag = ok ? 0 : 1;
        if (ok && nsl >= 0) issue_z(nsl);
      }
      __syncthreads();
      if (*abort_flag) break;
      if (nsl >= 0) {
        cm0 = msg_in[nin0 + e];
        cm1 = msg_in[nin1 + e];
        cnet = nnet;
      }
      continue;
    }

    MSG[q0] = cm0;
    MSG[q1] = cm1;
    __syncthreads();
    {
      // Kronecker products: threads 0-63 build K12 = M1 (x) M2, 64-127 K34 = M3 (x) M4;
      // row n = b_a + 8 b_b, column k = a_a + 8 a_b (16-byte chunk a_b), value M_a[b_a,a_a] M_b[b_b,a_b]
      const int n = t & 63, ba = n & 7, bb = n >> 3;
      const float* Ma = MSG + (t < 64 ? 0 : 128);
      const float* Mb = Ma + 64;
      float ma[8];
#pragma unroll
      for (int aa = 0; aa < 8; ++aa) ma[aa] = Ma[ba + 8 * aa];
      uint4* row = reinterpret_cast<uint4*>(KT + (t < 64 ? 0 : 8192) + n * 128);
#pragma unroll
      for (int ab = 0; ab < 8; ++ab) {
        const float mb = Mb[bb + 8 * ab];
        uint4 qv;
        qv.x = pack_bf16(ma[0] * mb, ma[1] * mb);
        qv.y = pack_bf16(ma[2] * mb, ma[3] * mb);
        qv.z = pack_bf16(ma[4] * mb, ma[5] * mb);
        qv.w = pack_bf16(ma[6] * mb, ma[7] * mb);
        row[ab ^ (n & 7)] = qv;
      }
      tc::fence_proxy_async_smem();
    }
    if (t == 0) *abort_flag = wait_z() ? 0 : 1;
    __syncthreads();
    if (*abort_flag) break;

    const uint32_t zaddr = tc::smem_u32(Z), ktaddr = tc::smem_u32(KT), t34addr = tc::smem_u32(T34);
    // ---- GEMM1 -> columns [0,64), GEMM1' -> [64,128) ----
    if (t == 0) {
      tc::tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(tmem + 0, tc::smem_desc(zaddr + 32 * kk, 16, 1024), tc::smem_desc(ktaddr + 32 * kk, 16, 1024),
                     kIdescG1, kk > 0);
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(tmem + 64, tc::smem_desc(zaddr + 2048 * kk, 8192, 1024),
                     tc::smem_desc(ktaddr + 8192 + 32 * kk, 16, 1024), kIdescG1mn, kk > 0);
      commit();
      *abort_flag = wait_mma() ? 0 : 1;
    }
    __syncthreads();
    if (*abort_flag) break;
    tc::tc_fence_after();
    {
      float d[32];
      tmem_ld_x32(trow + 0, d);
      store_half_row(KT, t, 0, d);  // T12 overwrites the Kronecker products (their MMAs are done)
      tmem_ld_x32(trow + 32, d);
      store_half_row(KT, t, 4, d);
      tmem_ld_x32(trow + 64, d);
      store_half_row(T34, t, 0, d);
      tmem_ld_x32(trow + 96, d);
      store_half_row(T34, t, 4, d);
    }
    tc::fence_proxy_async_smem();
    tc::tc_fence_before();
    __syncthreads();
    // ---- GEMM2 -> columns [0,128) ----
    if (t == 0) {
      tc::tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(tmem + 0, tc::smem_desc(ktaddr + 32 * kk, 16, 1024), tc::smem_desc(zaddr + 32 * kk, 16, 1024),
                     kIdescG2, kk > 0);
      commit();
      *abort_flag = wait_mma() ? 0 : 1;
    }
    // the next vertex's incoming messages, ahead of use
    if (nsl >= 0) {
      nm0 = msg_in[nin0 + e];
      nm1 = msg_in[nin1 + e];
    }
    __syncthreads();
    if (*abort_flag) break;
    tc::tc_fence_after();
    diag_to_env(trow, G, t);  // G34 (overwrites T12: GEMM2 is done)
    tc::tc_fence_before();
    __syncthreads();
    // ---- GEMM2' -> columns [0,128), overlapped with the G34 epilogue ----
    if (t == 0) {
      tc::tc_fence_after();
#pragma unroll
      for (int kk = 0; kk < 4; ++kk)
        tc::mma_bf16(tmem + 0, tc::smem_desc(t34addr + 32 * kk, 16, 1024),
                     tc::smem_desc(zaddr + 2048 * kk, 8192, 1024), kIdescG2mn, kk > 0);
      commit();
    }
    env_to_out(G, MSG + 192, MSG + 128, RES + 128, RES + 192, t);  // out3 (with M4), out4 (with M3)
    if (t == 0) {
      const bool ok = wait_mma();
      *abort_flag = ok ? 0 : 1;
      if (ok && nsl >= 0) issue_z(nsl);  // Z is free: fetch the next vertex's image
    }
    __syncthreads();
    if (*abort_flag) break;
    tc::tc_fence_after();
    diag_to_env(trow, G, t);  // G12
    env_to_out(G, MSG + 64, MSG, RES, RES + 64, t);  // out1 (with M2), out2 (with M1)
    tc::tc_fence_before();
    __syncthreads();
    {
      const double df = tc_finalize(RES + 64 * warp, msg_in + out_off_w, msg_out + out_off_w, normalize,
                                    want_diff != 0, lane);
      if (want_diff && lane == 0) diffs[out_de_w] = df;
    }
    cm0 = nm0;
    cm1 = nm1;
    cnet = nnet;
  }

  // drain: after a timeout, wait (bounded) for this CTA's own copy and MMAs
  if (t == 0 && *abort_flag) {
    atomicExch(err, (int)GBTN_ERR_TIMEOUT);
    if (tma_pending) wait_z();
    if (mma_pending) wait_mma();
  }
  tc::tc_fence_before();
  __syncthreads();
  tc::tc_fence_after();
  if (warp == 0) tc::tmem_dealloc(tmem, kTmemCols);
}

namespace {

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

}  // namespace

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

void launch_tc_vertices(const int* work, int nwork, const int* vslot, const TcRec* recs, const __nv_bfloat16* zimg,
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
  tc_vertex_kernel<<<grid, kTcThreads, kSmemBytes, s>>>(work, nwork, vslot, recs, zimg, msg_in, msg_out, diffs,
                                                         converged, normalize, want_diff, err);
  GBTN_CUDA(cudaGetLastError());
}

}  // namespace gbtn
