// Global-memory ("large vertex") message kernels: vertices whose tensors do
// not fit the shared-memory kernels -- bond dimensions 9..64, site dimensions
// 9..64, or tensors above the shared-memory budget -- with no limit from
// shared memory on the tensor size (the plan caps it at 2^28 elements).
//
// The same shared-prefix schedule as the shared-memory kernels
// (abstractbeliefpropagationcache.jl:225-239, every outgoing message of a
// vertex from its incoming messages) runs as one launch per schedule step over
// a wave of vertices of one degree; the intermediate tensors live in a
// scratch area in HBM (buffers 1..nbuf-1 of every wave vertex; buffer 0 is
// the site tensor itself):
//
//   ABSORB(src -> dst, leg p):  dst[.., b, ..] = sum_a M_p[b, a] src[.., a, ..]
//   CLOSE(src, leg p):          res[b, a] = sum_fibers conj(bra[.., b, ..]) src[.., a, ..]
//
// A fiber of leg p is the chi_p values at stride st_p; the fibers of a vertex
// are cut into tiles of at most kTile elements that are contiguous in memory
// (whole groups of st_p * chi_p elements when that fits, else runs of Lt
// consecutive fibers per leg index), so every tile is read and written with
// coalesced accesses and staged in shared memory.  ABSORB writes its tile's
// outputs directly; CLOSE writes one chi x chi partial sum per tile, and a
// finishing launch adds the partials of every tile in a fixed order
// (deterministic), normalises the message in FP64 and records message_diff
// (abstractbeliefpropagationcache.jl:32-36).  CLOSE on the site index (st = 1,
// chi = d) gives the one-site reduced density matrix (expect.jl:5-19).
//
// T is the arithmetic (double, float, df32, zdouble, zfloat), S the storage
// of tensors and messages (S = T, or double under df32).
#include "bp_device.cuh"

namespace gbtn {

namespace {

constexpr int kLargeThreads = 256;
constexpr int kCloseRed = 16 * kLargeThreads;  // CLOSE: one 4 x 4 block per thread and slice

__host__ __device__ inline long long lmin(long long a, long long b) { return a < b ? a : b; }

// complex view of an arithmetic element (re, im) in FP64
__device__ __forceinline__ void to_z(double x, double& r, double& i) { r = x; i = 0.0; }
__device__ __forceinline__ void to_z(float x, double& r, double& i) { r = x; i = 0.0; }
__device__ __forceinline__ void to_z(df32 x, double& r, double& i) { r = df_to_double(x); i = 0.0; }
__device__ __forceinline__ void to_z(zdouble x, double& r, double& i) { r = x.re; i = x.im; }
__device__ __forceinline__ void to_z(zfloat x, double& r, double& i) { r = x.re; i = x.im; }
template <typename S>
__device__ __forceinline__ S from_z(double r, double i);
template <> __device__ __forceinline__ double from_z<double>(double r, double) { return r; }
template <> __device__ __forceinline__ float from_z<float>(double r, double) { return (float)r; }
template <> __device__ __forceinline__ zdouble from_z<zdouble>(double r, double i) { return zdouble(r, i); }
template <> __device__ __forceinline__ zfloat from_z<zfloat>(double r, double i) { return zfloat((float)r, (float)i); }
// arithmetic element -> storage element
template <typename S, typename T>
__device__ __forceinline__ S from_elem(T x) {
  if constexpr (std::is_same<T, df32>::value)
    return df_to_double(x);
  else
    return x;
}

__device__ __forceinline__ double block_sum(double x, double* red) {
  x = warp_sum(x);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = x;
  __syncthreads();
  double t = 0.0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
  return t;
}

// Scratch buffer b (1..nbuf-1) of wave vertex w.
template <typename T>
__device__ __forceinline__ T* wave_buf(T* scratch, const long long* buf_off, int w, int b, int n) {
  return scratch + buf_off[w] + (long long)(b - 1) * n;
}

template <typename T, typename S>
__global__ void __launch_bounds__(kLargeThreads)
    large_absorb_kernel(LargeArgs<S> a, T* __restrict__ scratch, int src, int dst, int leg, const int* converged) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = blockIdx.y;
  const int v = a.verts[w];
  const VDesc& d = a.vd[v];
  if (converged && converged[d.net]) return;
  const int n = d.n, chi = d.chi[leg], st = d.st[leg];
  const LegTiling g = leg_tiling(n, st, chi);
  const int t = blockIdx.x;
  if (t >= g.ntl * g.ntj) return;
  T* M = reinterpret_cast<T*>(smem);
  T* tile = M + align_up((size_t)chi * chi, 4);
  const S* m = a.msgs + a.msg_off[d.in_de[leg]];
  for (int i = threadIdx.x; i < chi * chi; i += kLargeThreads) M[i] = to_elem<T>(m[i]);
  const int l0 = (t % g.ntl) * g.Lt;
  const long long j0 = (long long)(t / g.ntl) * g.R;
  const int nl = (int)lmin(g.Lt, st - l0);
  const int nj = (int)lmin(g.R, g.nouter - j0);
  const long long base = j0 * st * chi + l0;
  const int cnt = nj * chi * nl;
  if (src == 0) {
    const S* in = a.fac + d.a_off + base;
    for (int i = threadIdx.x; i < cnt; i += kLargeThreads) tile[i] = to_elem<T>(in[(long long)(i / nl) * st + i % nl]);
  } else {
    const T* in = wave_buf(scratch, a.buf_off, w, src, n) + base;
    for (int i = threadIdx.x; i < cnt; i += kLargeThreads) tile[i] = in[(long long)(i / nl) * st + i % nl];
  }
  __syncthreads();
  // four outputs b0 .. b0 + 3 of one fiber (j, l) per work item: each fiber
  // value is loaded once for the four; adjacent threads take adjacent l with
  // the same b0, so M is read by broadcast and the tile without conflicts
  T* out = wave_buf(scratch, a.buf_off, w, dst, n) + base;
  const int nb4 = (chi + 3) / 4;
  const int items = nj * nb4 * nl;
  for (int i = threadIdx.x; i < items; i += kLargeThreads) {
    const int l = i % nl, rest = i / nl, b0 = (rest % nb4) * 4, j = rest / nb4;
    const T* x = tile + (long long)j * chi * nl + l;
    T y[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) y[k] = T(0);
    for (int q = 0; q < chi; ++q) {
      const T xq = x[q * nl];
#pragma unroll
      for (int k = 0; k < 4; ++k)
        if (b0 + k < chi) y[k] = mac(M[b0 + k + chi * q], xq, y[k]);
    }
#pragma unroll
    for (int k = 0; k < 4; ++k)
      if (b0 + k < chi) out[((long long)j * chi + b0 + k) * st + l] = settle(y[k]);
  }
}

// One partial chi x chi CLOSE per tile: partial[w * vstride + t * P + o]
// (vstride: elements of partial sums reserved per wave vertex).
template <typename T, typename S>
__global__ void __launch_bounds__(kLargeThreads)
    large_close_kernel(LargeArgs<S> a, const T* __restrict__ scratch, int src, int leg, T* __restrict__ partial,
                       long long vstride, const int* converged) {
  extern __shared__ __align__(16) unsigned char smem[];
  const int w = blockIdx.y;
  const int v = a.verts[w];
  const VDesc& d = a.vd[v];
  if (converged && converged[d.net]) return;
  const int n = d.n;
  const int chi = leg >= 0 ? d.chi[leg] : d.d, st = leg >= 0 ? d.st[leg] : 1;
  const LegTiling g = leg_tiling(n, st, chi);
  const int t = blockIdx.x;
  if (t >= g.ntl * g.ntj) return;
  T* tt = reinterpret_cast<T*>(smem);
  T* tb = tt + kTile;
  T* red = tb + kTile;
  const int l0 = (t % g.ntl) * g.Lt;
  const long long j0 = (long long)(t / g.ntl) * g.R;
  const int nl = (int)lmin(g.Lt, st - l0);
  const int nj = (int)lmin(g.R, g.nouter - j0);
  const long long base = j0 * st * chi + l0;
  const int cnt = nj * chi * nl;
  const S* braw = (a.bra ? a.bra : a.fac) + d.a_off + base;
  if (src == 0) {
    const S* in = a.fac + d.a_off + base;
    for (int i = threadIdx.x; i < cnt; i += kLargeThreads) tt[i] = to_elem<T>(in[(long long)(i / nl) * st + i % nl]);
  } else {
    const T* in = wave_buf(scratch, a.buf_off, w, src, n) + base;
    for (int i = threadIdx.x; i < cnt; i += kLargeThreads) tt[i] = in[(long long)(i / nl) * st + i % nl];
  }
  for (int i = threadIdx.x; i < cnt; i += kLargeThreads)
    tb[i] = conj_of(to_elem<T>(braw[(long long)(i / nl) * st + i % nl]));
  __syncthreads();
  // res[b, q] = sum over the tile's fibers f of bra[f, b] ket[f, q]: a small
  // GEMM.  A thread accumulates a 4 x 4 block (b0.., q0..) over the fibers
  // f = s, s + NS, ... of its slice s (8 loads per 16 multiply-adds; adjacent
  // threads take adjacent fibers, so the loads do not conflict); the slices are
  // then added in slice order (deterministic).  Blocks are taken `groups` at a
  // time when there are more than the threads' share.
  const int P = chi * chi;
  const int nf = nj * nl;  // fibers of the tile: (j, l)
  const int nbb = (chi + 3) / 4, nblk = nbb * nbb;
  const int NS = nblk >= kLargeThreads ? 1 : kLargeThreads / nblk;  // fiber slices
  const int groups = kLargeThreads / NS;                           // blocks per pass
  T* out = partial + (long long)w * vstride + (long long)t * P;
  for (int bk0 = 0; bk0 < nblk; bk0 += groups) {
    const int sl = threadIdx.x % NS, gb = threadIdx.x / NS, bk = bk0 + gb;
    T acc[4][4];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
      for (int k = 0; k < 4; ++k) acc[i][k] = T(0);
    if (gb < groups && bk < nblk) {
      const int b0 = (bk % nbb) * 4, q0 = (bk / nbb) * 4;
      for (int f = sl; f < nf; f += NS) {
        const int j = f / nl, l = f % nl;
        const long long row = (long long)j * chi * nl + l;
        T yb[4], xq[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
          yb[i] = b0 + i < chi ? tb[row + (long long)(b0 + i) * nl] : T(0);
          xq[i] = q0 + i < chi ? tt[row + (long long)(q0 + i) * nl] : T(0);
        }
#pragma unroll
        for (int i = 0; i < 4; ++i)
#pragma unroll
          for (int k = 0; k < 4; ++k) acc[i][k] = mac(yb[i], xq[k], acc[i][k]);
      }
#pragma unroll
      for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int k = 0; k < 4; ++k) red[((long long)sl * groups + gb) * 16 + i * 4 + k] = settle(acc[i][k]);
    }
    __syncthreads();
    for (int o = threadIdx.x; o < groups * 16; o += kLargeThreads) {
      const int g = o / 16, e = o % 16, bkk = bk0 + g;
      if (bkk >= nblk) continue;
      const int b = (bkk % nbb) * 4 + e / 4, q = (bkk / nbb) * 4 + e % 4;
      if (b >= chi || q >= chi) continue;
      T sum = T(0);
      for (int s2 = 0; s2 < NS; ++s2) sum += red[((long long)s2 * groups + g) * 16 + e];
      out[b + chi * q] = sum;
    }
    __syncthreads();
  }
}

// Sum of the tile partials of wave vertex w, output o, in tile order.
template <typename T>
__device__ __forceinline__ T sum_partials(const T* partial, int w, long long vstride, int tiles, int P, int o) {
  T s = T(0);
  const T* p = partial + (long long)w * vstride + o;
  for (int t = 0; t < tiles; ++t) s += p[(long long)t * P];
  return s;
}

// Outgoing message on `leg` of every wave vertex: partial sums added, FP64
// normalisation, message_diff against the old message, stored as S.
template <typename T, typename S>
__global__ void __launch_bounds__(kLargeThreads)
    large_finish_msg_kernel(LargeArgs<S> a, const T* __restrict__ partial, long long vstride, int leg, const S* msg_old,
                            S* msg_out, double* diffs, const int* converged, int normalize, int want_diff) {
  __shared__ double red[kLargeThreads / 32];
  const int w = blockIdx.x;
  const int v = a.verts[w];
  const VDesc& d = a.vd[v];
  const int chi = d.chi[leg], P = chi * chi;
  const int de = d.out_de[leg];
  const long long off = a.msg_off[de];
  if (converged && converged[d.net]) {
    if (msg_old != msg_out)
      for (int o = threadIdx.x; o < P; o += kLargeThreads) msg_out[off + o] = msg_old[off + o];
    return;
  }
  const LegTiling g = leg_tiling(d.n, d.st[leg], chi);
  const int tiles = g.ntl * g.ntj;
  double nr2 = 0.0, dre = 0.0, dim = 0.0, nb = 0.0;
  for (int o = threadIdx.x; o < P; o += kLargeThreads) {
    double r, i, orr, oi;
    to_z(sum_partials(partial, w, vstride, tiles, P, o), r, i);
    to_z(msg_old[off + o], orr, oi);
    nr2 += r * r + i * i;
    dre += orr * r + oi * i;  // <old, new> = sum conj(old) new
    dim += orr * i - oi * r;
    nb += orr * orr + oi * oi;
  }
  nr2 = block_sum(nr2, red);
  dre = block_sum(dre, red);
  dim = block_sum(dim, red);
  nb = block_sum(nb, red);
  const double sc = (normalize && nr2 > 0.0) ? 1.0 / sqrt(nr2) : 1.0;
  __syncthreads();  // every old entry is read before any is overwritten (in-place schedules)
  for (int o = threadIdx.x; o < P; o += kLargeThreads) {
    double r, i;
    to_z(sum_partials(partial, w, vstride, tiles, P, o), r, i);
    msg_out[off + o] = from_z<S>(r * sc, i * sc);
  }
  if (want_diff && threadIdx.x == 0) diffs[de] = 1.0 - (dre * dre + dim * dim) / (nr2 * nb);
}

// One-site reduced density matrix rho[s', s] of every wave vertex.
template <typename T, typename S>
__global__ void __launch_bounds__(kLargeThreads)
    large_finish_rdm_kernel(LargeArgs<S> a, const T* __restrict__ partial, long long vstride, S* rdm,
                            const long long* rdm_off) {
  const int w = blockIdx.x;
  const int v = a.verts[w];
  const VDesc& d = a.vd[v];
  const int P = d.d * d.d;
  const LegTiling g = leg_tiling(d.n, 1, d.d);
  const int tiles = g.ntl * g.ntj;
  for (int o = threadIdx.x; o < P; o += kLargeThreads)
    rdm[rdm_off[v] + o] = from_elem<S>(sum_partials(partial, w, vstride, tiles, P, o));
}

}  // namespace

template <typename T, typename S>
void launch_large_op(const LargeArgs<S>& a, int nverts, int max_tiles, int max_chi, const SchedOp& op, void* scratch_v,
                     void* partial_v, long long vstride, const S* msg_old, S* msg_out, double* diffs, const int* converged,
                     int normalize, int want_diff, cudaStream_t s) {
  if (nverts == 0) return;
  T* scratch = static_cast<T*>(scratch_v);
  T* partial = static_cast<T*>(partial_v);
  const dim3 grid(max_tiles, nverts);
  if (op.type == 0) {
    const size_t sm = sizeof(T) * (align_up((size_t)max_chi * max_chi, 4) + kTile);
    GBTN_CUDA(cudaFuncSetAttribute(large_absorb_kernel<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    large_absorb_kernel<T, S><<<grid, kLargeThreads, sm, s>>>(a, scratch, op.src, op.dst, op.leg, converged);
  } else {
    const size_t sm = sizeof(T) * (2 * (size_t)kTile + kCloseRed);
    GBTN_CUDA(cudaFuncSetAttribute(large_close_kernel<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    large_close_kernel<T, S><<<grid, kLargeThreads, sm, s>>>(a, scratch, op.src, op.leg, partial, vstride, converged);
    GBTN_CUDA(cudaGetLastError());
    large_finish_msg_kernel<T, S><<<nverts, kLargeThreads, 0, s>>>(a, partial, vstride, op.leg, msg_old, msg_out,
                                                                    diffs, converged, normalize, want_diff);
  }
  GBTN_CUDA(cudaGetLastError());
}

template <typename T, typename S>
void launch_large_rdm(const LargeArgs<S>& a, int nverts, int max_tiles, int src, void* scratch_v, void* partial_v,
                      long long vstride, S* rdm, const long long* rdm_off, cudaStream_t s) {
  if (nverts == 0) return;
  T* scratch = static_cast<T*>(scratch_v);
  T* partial = static_cast<T*>(partial_v);
  const size_t sm = sizeof(T) * (2 * (size_t)kTile + kCloseRed);
  GBTN_CUDA(cudaFuncSetAttribute(large_close_kernel<T, S>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  large_close_kernel<T, S><<<dim3(max_tiles, nverts), kLargeThreads, sm, s>>>(a, scratch, src, -1, partial, vstride,
                                                                               nullptr);
  GBTN_CUDA(cudaGetLastError());
  large_finish_rdm_kernel<T, S><<<nverts, kLargeThreads, 0, s>>>(a, partial, vstride, rdm, rdm_off);
  GBTN_CUDA(cudaGetLastError());
}

void launch_large_op_any(int arith, const LargeArgs<double>& ad, int nverts, int max_tiles, int max_chi,
                         const SchedOp& op, void* scratch, void* partial, long long vstride, const void* msg_old,
                         void* msg_out, double* diffs, const int* converged, int normalize, int want_diff,
                         cudaStream_t s) {
  const auto& af = reinterpret_cast<const LargeArgs<float>&>(ad);
  const auto& az = reinterpret_cast<const LargeArgs<zdouble>&>(ad);
  const auto& azf = reinterpret_cast<const LargeArgs<zfloat>&>(ad);
  switch (arith) {
    case kArithF64:
      launch_large_op<double, double>(ad, nverts, max_tiles, max_chi, op, scratch, partial, vstride,
                                      static_cast<const double*>(msg_old), static_cast<double*>(msg_out), diffs,
                                      converged, normalize, want_diff, s);
      break;
    case kArithF32:
      launch_large_op<float, float>(af, nverts, max_tiles, max_chi, op, scratch, partial, vstride,
                                    static_cast<const float*>(msg_old), static_cast<float*>(msg_out), diffs,
                                    converged, normalize, want_diff, s);
      break;
    case kArithDF32:
      launch_large_op<df32, double>(ad, nverts, max_tiles, max_chi, op, scratch, partial, vstride,
                                    static_cast<const double*>(msg_old), static_cast<double*>(msg_out), diffs,
                                    converged, normalize, want_diff, s);
      break;
    case kArithZ64:
      launch_large_op<zdouble, zdouble>(az, nverts, max_tiles, max_chi, op, scratch, partial, vstride,
                                        static_cast<const zdouble*>(msg_old), static_cast<zdouble*>(msg_out), diffs,
                                        converged, normalize, want_diff, s);
      break;
    case kArithZ32:
      launch_large_op<zfloat, zfloat>(azf, nverts, max_tiles, max_chi, op, scratch, partial, vstride,
                                      static_cast<const zfloat*>(msg_old), static_cast<zfloat*>(msg_out), diffs,
                                      converged, normalize, want_diff, s);
      break;
    default:
      throw std::logic_error("large path: unknown arithmetic");
  }
}

void launch_large_rdm_any(int arith, const LargeArgs<double>& ad, int nverts, int max_tiles, int src, void* scratch,
                          void* partial, long long vstride, void* rdm, const long long* rdm_off, cudaStream_t s) {
  if (arith == kArithZ64)
    launch_large_rdm<zdouble, zdouble>(reinterpret_cast<const LargeArgs<zdouble>&>(ad), nverts, max_tiles, src,
                                       scratch, partial, vstride, static_cast<zdouble*>(rdm), rdm_off, s);
  else if (arith == kArithF64)
    launch_large_rdm<double, double>(ad, nverts, max_tiles, src, scratch, partial, vstride, static_cast<double*>(rdm),
                                     rdm_off, s);
  else
    throw std::logic_error("large path: environments are FP64 or complex FP64");
}

size_t large_elem_size(int arith) {
  switch (arith) {
    case kArithF32: return sizeof(float);
    case kArithZ64: return sizeof(zdouble);
    case kArithZ32: return sizeof(zfloat);
    default: return 8;  // double, df32
  }
}

}  // namespace gbtn
