// SIMT kernels of the belief-propagation hot path (FP64 and FP32 arithmetic).
//
// A vertex v of the quadratic-form network <psi|psi> holds the ket tensor
// A_v[s, a_1..a_k] (column-major); the bra is conj(A_v) (or a separate bra
// tensor).  Every kernel here is built from two shared-memory "fiber" steps:
//
//   ABSORB(src -> dst, leg p):  dst[.., b_p, ..] = sum_a M_p[b_p, a] src[.., a, ..]
//     (the incoming message on leg p moves the ket index a_p to the bra index b_p)
//   CLOSE(src, leg p):          out[b, a] = sum_{fibers} bra[.., b, ..] * src[.., a, ..]
//     (all other legs of src already carry bra indices; the site index is shared)
//
// The outgoing message on leg p (updated_message,
// src/caches/abstractbeliefpropagationcache.jl:225-239) is CLOSE(p) of the
// tensor with every other incoming message absorbed; all k outgoing messages
// of a vertex share absorbed prefixes through a host-built schedule
// (12 instead of 16 contraction steps at degree 4).  CLOSE on the site leg
// gives the one-site reduced density matrix (expect.jl:5-19).
#include <cmath>
#include <functional>
#include <numeric>

#include "bp_device.cuh"

namespace gbtn {

__constant__ DeviceSched c_sched;

// ---------------------------------------------------------------------------
// Host: vertex schedules
// ---------------------------------------------------------------------------

DeviceSched build_schedules() {
  DeviceSched s{};
  for (int k = 0; k <= kMaxDeg; ++k) {
    std::vector<SchedOp> ops;
    int maxbuf = 0;
    std::function<void(int, const std::vector<int>&, const std::vector<int>&)> gen =
        [&](int src, const std::vector<int>& W, const std::vector<int>& freeb) {
          if (W.size() == 1) {
            ops.push_back({1, (int8_t)src, 0, (int8_t)W[0]});
            return;
          }
          const size_t h = W.size() / 2;
          std::vector<int> W1(W.begin(), W.begin() + h), W2(W.begin() + h, W.end());
          for (int half = 0; half < 2; ++half) {
            const std::vector<int>& keep = half == 0 ? W1 : W2;
            const std::vector<int>& absorb = half == 0 ? W2 : W1;
            int cur = src;
            for (int leg : absorb) {
              int dst = -1;
              for (int b : freeb)
                if (b != cur) {
                  dst = b;
                  break;
                }
              if (dst < 0) throw std::logic_error("schedule: out of buffers");
              ops.push_back({0, (int8_t)cur, (int8_t)dst, (int8_t)leg});
              maxbuf = std::max(maxbuf, dst);
              cur = dst;
            }
            std::vector<int> fb2;
            for (int b : freeb)
              if (b != cur) fb2.push_back(b);
            gen(cur, keep, fb2);
          }
        };
    if (k >= 1) {
      std::vector<int> W(k);
      std::iota(W.begin(), W.end(), 0);
      std::vector<int> freeb;
      for (int b = 1; b < kNumBufs; ++b) freeb.push_back(b);
      gen(0, W, freeb);
    }
    if ((int)ops.size() > kMaxOps) throw std::logic_error("schedule too long");
    for (size_t i = 0; i < ops.size(); ++i) s.ops[k][i] = ops[i];
    s.len[k] = (int)ops.size();
    s.nbuf[k] = maxbuf + 1;
  }
  return s;
}

void upload_schedules(const DeviceSched& s) { GBTN_CUDA(cudaMemcpyToSymbol(c_sched, &s, sizeof(s))); }

// ---------------------------------------------------------------------------
// Jacobi / coloured sweep kernel: every listed vertex computes all of its
// outgoing messages from msg_in into msg_out.
// ---------------------------------------------------------------------------

// T is the arithmetic, S the storage in HBM (S = T, or double for the
// double-FP32 refinement sweeps, whose tensors and messages stay FP64).
template <typename T, int TEAM, typename S = T>
__global__ void __launch_bounds__(TEAM == 32 ? 128 : TEAM)
    bp_vertex_kernel(const int* __restrict__ work, int nwork, const VDesc* __restrict__ vd,
                     const S* __restrict__ fac, const S* __restrict__ bra_g, const S* msg_in, S* msg_out,
                     const long long* __restrict__ msg_off, double* diffs, const int* converged,
                     int normalize, int want_diff, int ncap, int nbuf) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPB = TEAM == 32 ? 4 : 1;
  const int team = threadIdx.x / TEAM, tid = threadIdx.x % TEAM, lane = tid & 31;
  const size_t tb = team_smem_bytes<T>(padded_len(ncap), nbuf, bra_g != nullptr, TEAM);
  TeamSmem<T> Sm = carve<T>(smem_raw + team * tb, padded_len(ncap), nbuf, bra_g != nullptr, TEAM);
  for (int w = blockIdx.x * TPB + team; w < nwork; w += gridDim.x * TPB) {
    const int v = work[w];
    load_desc<TEAM>(Sm.desc, vd + v, tid);
    tsync<TEAM>();
    const VDesc& d = *Sm.desc;
    if (converged && converged[d.net]) {
      if (msg_in != msg_out) {
        for (int p = 0; p < d.k; ++p) {
          const long long off = msg_off[d.out_de[p]];
          const int c2 = d.chi[p] * d.chi[p];
          for (int i = tid; i < c2; i += TEAM) msg_out[off + i] = msg_in[off + i];
        }
      }
      tsync<TEAM>();
      continue;
    }
    load_vertex<T, TEAM, S, true>(Sm, fac, bra_g, msg_in, msg_off, -1, tid);
    if (want_diff) load_old_messages<T, TEAM, S>(Sm, msg_in, msg_off, tid);
    tsync<TEAM>();
    const int k = d.k;
    const int len = c_sched.len[k];
    // normalise leg p's close result, write it, and record message_diff against Sm.old
    auto finalize = [&](int p, const T* res) {
      const int de = d.out_de[p];
      const long long off = msg_off[de];
      const S* old = reinterpret_cast<const S*>(Sm.old) + p * 64;
      double df;
      if constexpr (std::is_same<T, df32>::value)
        df = finalize_message_df(res, d.chi[p], old, msg_out + off, normalize, want_diff != 0, lane);
      else
        df = finalize_message<T>(res, d.chi[p], old, msg_out + off, normalize, want_diff != 0, lane);
      if (want_diff && lane == 0) diffs[de] = df;
    };
    for (int i = 0; i < len; ++i) {
      const SchedOp op = c_sched.ops[k][i];
      const int leg = op.leg;
      const int chi = d.chi[leg], st = d.st[leg];
      if (op.type == 0) {
        absorb_any<T, true, TEAM == 32>(chi, Sm.buf[op.src], Sm.buf[op.dst], d.n, st, Sm.msg + leg * 64, tid, TEAM);
        tsync<TEAM>();
      } else if constexpr (TEAM > 32) {
        // the result waits in its leg's slot; close_fibers ends with a team barrier
        close_any<T, TEAM, true>(chi, Sm.buf[op.src], Sm.bra, d.n, st, 1, 0, 0, Sm.red, Sm.res + leg * 64, tid);
      } else {
        close_any<T, TEAM, true, true>(chi, Sm.buf[op.src], Sm.bra, d.n, st, 1, 0, 0, Sm.red, Sm.res, tid);
        finalize(leg, Sm.res);
        tsync<TEAM>();
      }
    }
    if constexpr (TEAM > 32) {
      // every leg's message at once, one warp each
      for (int p = tid >> 5; p < k; p += TEAM / 32) finalize(p, Sm.res + p * 64);
      tsync<TEAM>();
    }
  }
}

// ---------------------------------------------------------------------------
// Sequential schedule: waves of messages that do not depend on one another,
// each update seeing every earlier one; convergence is tested on the device
// after every sweep (abstractbeliefpropagationcache.jl:272-287,313-329).
// ---------------------------------------------------------------------------

// Compute the message leaving v on leg p from the loaded vertex: absorb every
// other leg (ping-pong through buffers 1 and 2), then CLOSE on p.
template <typename T, int TEAM>
__device__ __forceinline__ int chain_absorb(const TeamSmem<T>& S, int skip_leg, int tid) {
  const VDesc& d = *S.desc;
  int cur = 0;
  for (int j = 0; j < d.k; ++j) {
    if (j == skip_leg) continue;
    const int nxt = cur == 1 ? 2 : 1;
    absorb_any<T, true>(d.chi[j], S.buf[cur], S.buf[nxt], d.n, d.st[j], S.msg + j * 64, tid, TEAM);
    tsync<TEAM>();
    cur = nxt;
  }
  return cur;
}

// ---------------------------------------------------------------------------
// Block-sparse (U(1)-graded) networks: one job per nonzero sector block of a
// vertex tensor.  Messages of a charge-conserving network stay block-diagonal
// in the link sectors (flux zero), so absorbing them keeps every leg of a
// block in its sector, and the bra block that closes a block has the same
// sectors as the ket block.  A block's share of the outgoing message on leg p
// (sector sigma_p) is therefore the dense update of the block alone, with the
// sector blocks of its incoming messages; the shares of all blocks with the
// same sector are added by qn_finalize (bp_qn.cu), which then normalises the
// whole message.  Block descriptor fields: a_off / n / d / k / chi / st as a
// vertex (d = site-sector dimension, chi = sector dimensions), in_de[p] = the
// incoming (directed edge, sector) message id, out_de[p] = the block's
// partial slot for leg p, net = its reduced-density-matrix slot.
// mode 0: every outgoing share (the shared-prefix schedule); mode 1: the
// block's share of rho_v (all legs absorbed, CLOSE on the site index).
// ---------------------------------------------------------------------------
// T is the arithmetic, S the storage of blocks, messages and shares (S = T,
// or double under double-FP32 arithmetic).
template <typename T, int TEAM, typename S = T>
__global__ void __launch_bounds__(TEAM == 32 ? 128 : 256)
    qn_block_kernel(const int* __restrict__ work, int nwork, const VDesc* __restrict__ bd,
                    const S* __restrict__ blocks, const S* __restrict__ msg_in,
                    const long long* __restrict__ sec_off, S* __restrict__ partial,
                    const long long* __restrict__ part_off, int mode, int ncap, int nbuf) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPB = TEAM == 32 ? 4 : 1;
  const int team = threadIdx.x / TEAM, tid = threadIdx.x % TEAM;
  const size_t tb = team_smem_bytes<T>(padded_len(ncap), nbuf, false, TEAM);
  TeamSmem<T> Sm = carve<T>(smem_raw + team * tb, padded_len(ncap), nbuf, false, TEAM);
  auto store = [](T x) -> S {
    if constexpr (std::is_same<T, df32>::value)
      return df_to_double(x);
    else
      return x;
  };
  for (int w = blockIdx.x * TPB + team; w < nwork; w += gridDim.x * TPB) {
    load_desc<TEAM>(Sm.desc, bd + work[w], tid);
    tsync<TEAM>();
    const VDesc& d = *Sm.desc;
    load_vertex<T, TEAM, S, true>(Sm, blocks, nullptr, msg_in, sec_off, -1, tid);
    tsync<TEAM>();
    if (mode == 1) {
      const int cur = chain_absorb<T, TEAM>(Sm, -1, tid);
      close_any<T, TEAM, true>(d.d, Sm.buf[cur], Sm.bra, d.n, 1, 1, 0, 0, Sm.red, Sm.res, tid);
      S* out = partial + part_off[d.net];
      for (int i = tid; i < d.d * d.d; i += TEAM) out[i] = store(Sm.res[i]);
      tsync<TEAM>();
      continue;
    }
    const int k = d.k;
    const int len = c_sched.len[k];
    for (int i = 0; i < len; ++i) {
      const SchedOp op = c_sched.ops[k][i];
      const int leg = op.leg;
      const int chi = d.chi[leg], st = d.st[leg];
      if (op.type == 0) {
        absorb_any<T, true>(chi, Sm.buf[op.src], Sm.buf[op.dst], d.n, st, Sm.msg + leg * 64, tid, TEAM);
        tsync<TEAM>();
      } else {
        close_any<T, TEAM, true>(chi, Sm.buf[op.src], Sm.bra, d.n, st, 1, 0, 0, Sm.red, Sm.res, tid);
        S* out = partial + part_off[d.out_de[leg]];
        for (int j = tid; j < chi * chi; j += TEAM) out[j] = store(Sm.res[j]);
        tsync<TEAM>();
      }
    }
  }
}

template <typename T, typename S>
void launch_qn_blocks_t(const WorkList& wl_all, const VDesc* bd, const S* blocks, const S* msg_in,
                        const long long* sec_off, S* partial, const long long* part_off, int mode, cudaStream_t s) {
  for (int c = 0; c < wl_all.nsubs(); ++c) {
    const WorkList wl = wl_all.sub(c);
    if (wl.count == 0) continue;
    const int nbuf = wl.maxdeg <= 4 ? 3 : kNumBufs;
    if (wl.team == 32) {
      const size_t sm = 4 * team_smem_bytes<T>(padded_len(wl.ncap), nbuf, false, 32);
      auto kern = qn_block_kernel<T, 32, S>;
      GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      kern<<<(wl.count + 3) / 4, 128, sm, s>>>(wl.d_vertices, wl.count, bd, blocks, msg_in, sec_off, partial, part_off,
                                               mode, wl.ncap, nbuf);
    } else {
      const size_t sm = team_smem_bytes<T>(padded_len(wl.ncap), nbuf, false, 256);
      auto kern = qn_block_kernel<T, 256, S>;
      GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
      kern<<<wl.count, 256, sm, s>>>(wl.d_vertices, wl.count, bd, blocks, msg_in, sec_off, partial, part_off, mode,
                                     wl.ncap, nbuf);
    }
    GBTN_CUDA(cudaGetLastError());
  }
}

void launch_qn_blocks(const WorkList& wl_all, const VDesc* bd, const double* blocks, const double* msg_in,
                      const long long* sec_off, double* partial, const long long* part_off, int mode,
                      cudaStream_t s) {
  launch_qn_blocks_t<double, double>(wl_all, bd, blocks, msg_in, sec_off, partial, part_off, mode, s);
}

void launch_qn_blocks_f32(const WorkList& wl_all, const VDesc* bd, const float* blocks, const float* msg_in,
                          const long long* sec_off, float* partial, const long long* part_off, cudaStream_t s) {
  launch_qn_blocks_t<float, float>(wl_all, bd, blocks, msg_in, sec_off, partial, part_off, 0, s);
}

void launch_qn_blocks_df32(const WorkList& wl_all, const VDesc* bd, const double* blocks, const double* msg_in,
                           const long long* sec_off, double* partial, const long long* part_off, cudaStream_t s) {
  launch_qn_blocks_t<df32, double>(wl_all, bd, blocks, msg_in, sec_off, partial, part_off, 0, s);
}

// One wave of the sequential schedule: every job (vertex, leg, sequence
// position, network) computes one message in place from the current messages
// (absorb chain of the other legs, CLOSE on the leg, normalisation) and
// records its message_diff at its sequence position.  The host cuts the
// sequence into waves so that no job of a wave reads or writes a message that
// another job of the same wave writes, and every job comes after the jobs it
// depends on in sequence order (read-after-write, write-after-read and
// write-after-write on the messages): the waves in order give the strictly
// sequential result (abstractbeliefpropagationcache.jl:272-287).
template <typename T, int TEAM, typename S = T>
__global__ void __launch_bounds__(TEAM == 32 ? 128 : 256)
    bp_wave_kernel(const int4* __restrict__ jobs, int njobs, const VDesc* __restrict__ vd, const S* __restrict__ fac,
                   const S* __restrict__ bra_g, S* msgs, const long long* __restrict__ msg_off, double* pos_diffs,
                   const int* converged, int normalize, int want_diff, int ncap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPB = TEAM == 32 ? 4 : 1;
  const int team = threadIdx.x / TEAM, tid = threadIdx.x % TEAM, lane = tid & 31;
  const size_t tb = team_smem_bytes<T>(padded_len(ncap), 3, bra_g != nullptr, TEAM);
  TeamSmem<T> Sm = carve<T>(smem_raw + team * tb, padded_len(ncap), 3, bra_g != nullptr, TEAM);
  for (int w = blockIdx.x * TPB + team; w < njobs; w += gridDim.x * TPB) {
    const int4 jb = jobs[w];  // (vertex, leg, sequence position, network)
    if (converged && converged[jb.w]) continue;  // uniform over the team
    load_desc<TEAM>(Sm.desc, vd + jb.x, tid);
    tsync<TEAM>();
    load_vertex<T, TEAM, S, true>(Sm, fac, bra_g, msgs, msg_off, jb.y, tid);
    tsync<TEAM>();
    const int cur = chain_absorb<T, TEAM>(Sm, jb.y, tid);
    const VDesc& d = *Sm.desc;
    const int chi = d.chi[jb.y];
    close_any<T, TEAM, true>(chi, Sm.buf[cur], Sm.bra, d.n, d.st[jb.y], 1, 0, 0, Sm.red, Sm.res, tid);
    if (tid < 32) {
      S* m = msgs + msg_off[d.out_de[jb.y]];
      double df;
      if constexpr (std::is_same<T, df32>::value)
        df = finalize_message_df(Sm.res, chi, m, m, normalize, want_diff != 0, lane);
      else
        df = finalize_message<T>(Sm.res, chi, m, m, normalize, want_diff != 0, lane);
      if (want_diff && lane == 0) pos_diffs[jb.z] = df;
    }
    tsync<TEAM>();
  }
}

// One message, FP64, written to out without touching the cache.
template <typename T>
__global__ void __launch_bounds__(256)
    updated_message_kernel(const VDesc* __restrict__ vd, int v, int leg, const T* __restrict__ fac,
                           const T* __restrict__ bra_g, const T* msgs, const long long* msg_off, T* out,
                           int ncap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TEAM = 256;
  const int tid = threadIdx.x;
  TeamSmem<T> S = carve<T>(smem_raw, padded_len(ncap), 3, bra_g != nullptr, TEAM);
  load_desc<TEAM>(S.desc, vd + v, tid);
  __syncthreads();
  load_vertex<T, TEAM, T, true>(S, fac, bra_g, msgs, msg_off, leg, tid);
  __syncthreads();
  const int cur = chain_absorb<T, TEAM>(S, leg, tid);
  const VDesc& d = *S.desc;
  close_any<T, TEAM, true>(d.chi[leg], S.buf[cur], S.bra, d.n, d.st[leg], 1, 0, 0, S.red, S.res, tid);
  if (tid < 32) finalize_message<T>(S.res, d.chi[leg], out, out, 1, false, tid);
}

// ---------------------------------------------------------------------------
// Environment kernels (FP64)
// ---------------------------------------------------------------------------

// rho_v[s', s] for every listed vertex: absorb all incoming messages, CLOSE on
// the site index.
// rho_v of every listed vertex: all incoming messages absorbed, CLOSE on the
// site index.  T is the arithmetic, S the storage (S = T, or double under
// df32 arithmetic: FP64 tensors, messages and RDMs, ~48-bit contractions).
template <typename T, int TEAM, typename S = T>
__global__ void __launch_bounds__(TEAM == 32 ? 128 : 256)
    vertex_rdm_kernel(const int* __restrict__ work, int nwork, const VDesc* __restrict__ vd,
                      const S* __restrict__ fac, const S* __restrict__ bra_g, const S* msgs,
                      const long long* __restrict__ msg_off, const long long* __restrict__ rdm_off, S* rdm,
                      int ncap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TPB = TEAM == 32 ? 4 : 1;
  const int team = threadIdx.x / TEAM, tid = threadIdx.x % TEAM;
  const size_t tb = team_smem_bytes<T>(padded_len(ncap), 3, bra_g != nullptr, TEAM);
  TeamSmem<T> Sm = carve<T>(smem_raw + team * tb, padded_len(ncap), 3, bra_g != nullptr, TEAM);
  for (int w = blockIdx.x * TPB + team; w < nwork; w += gridDim.x * TPB) {
    const int v = work[w];
    load_desc<TEAM>(Sm.desc, vd + v, tid);
    tsync<TEAM>();
    load_vertex<T, TEAM, S, true>(Sm, fac, bra_g, msgs, msg_off, -1, tid);
    tsync<TEAM>();
    const int cur = chain_absorb<T, TEAM>(Sm, -1, tid);
    const VDesc& d = *Sm.desc;
    close_any<T, TEAM, true>(d.d, Sm.buf[cur], Sm.bra, d.n, 1, 1, 0, 0, Sm.red, Sm.res, tid);
    for (int i = tid; i < d.d * d.d; i += TEAM) {
      if constexpr (std::is_same<T, df32>::value)
        rdm[rdm_off[v] + i] = df_to_double(Sm.res[i]);
      else
        rdm[rdm_off[v] + i] = Sm.res[i];
    }
    tsync<TEAM>();
  }
}

// Half of a two-site RDM: for job (v, p), R[s', s, b, a] with every incoming
// message of v except the one on leg p absorbed, stored at
// half[(s' + d*s)*chi*chi + b + chi*a].
template <typename T>
__global__ void __launch_bounds__(256)
    edge_half_kernel(const int2* __restrict__ jobs, int njobs, const VDesc* __restrict__ vd,
                     const T* __restrict__ fac, const T* __restrict__ bra_g, const T* msgs,
                     const long long* __restrict__ msg_off, T* halves, const long long* __restrict__ half_off,
                     int ncap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TEAM = 256;
  const int tid = threadIdx.x;
  TeamSmem<T> S = carve<T>(smem_raw, padded_len(ncap), 3, bra_g != nullptr, TEAM);
  for (int j = blockIdx.x; j < njobs; j += gridDim.x) {
    const int2 jb = jobs[j];
    load_desc<TEAM>(S.desc, vd + jb.x, tid);
    __syncthreads();
    load_vertex<T, TEAM, T, true>(S, fac, bra_g, msgs, msg_off, jb.y, tid);
    __syncthreads();
    const int cur = chain_absorb<T, TEAM>(S, jb.y, tid);
    const VDesc& d = *S.desc;
    const int chi = d.chi[jb.y];
    for (int s = 0; s < d.d; ++s)
      for (int sp = 0; sp < d.d; ++sp) {
        close_any<T, TEAM, true>(chi, S.buf[cur], S.bra, d.n, d.st[jb.y], d.d, s, sp - s, S.red, S.res, tid);
        for (int i = tid; i < chi * chi; i += TEAM) halves[half_off[j] + (long long)(sp + d.d * s) * chi * chi + i] = S.res[i];
        __syncthreads();
      }
  }
}

// ---------------------------------------------------------------------------
// Small elementwise / per-edge kernels
// ---------------------------------------------------------------------------

// Per network: mean message diff of the sweep, iteration count, convergence
// flag (mean <= tol).  With stall > 0 a network also stops when its mean diff
// has not dropped below 0.9x its best value for `stall` sweeps -- the noise
// floor of a reduced-precision phase.
__global__ void reduce_diffs_kernel(const int* __restrict__ net_de_ptr, const int* __restrict__ net_de,
                                    const double* __restrict__ diffs, double tol, int* converged, int* iters,
                                    double* mean_diff, int stall, double* best, int* since, int* n_conv) {
  const int net = blockIdx.x;
  if (converged[net]) return;
  const int b = net_de_ptr[net], e = net_de_ptr[net + 1];
  double s = 0.0;
  for (int i = b + threadIdx.x; i < e; i += blockDim.x) s += diffs[net_de[i]];
  __shared__ double red[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x < 32) {
    double t = threadIdx.x < (int)(blockDim.x >> 5) ? red[threadIdx.x] : 0.0;
    t = warp_sum(t);
    if (threadIdx.x == 0) {
      const double mean = t / (double)(e - b);
      iters[net] += 1;
      mean_diff[net] = tol >= 0.0 ? mean : NAN;
      int done = tol >= 0.0 && mean <= tol;
      if (stall > 0) {
        if (iters[net] == 1 || mean < 0.9 * best[net]) {
          best[net] = mean;
          since[net] = 0;
        } else if (++since[net] >= stall) {
          done = 1;
        }
      }
      if (done) {
        converged[net] = 1;
        if (n_conv) atomicAdd(n_conv, 1);  // the host stops the sweeps once every network is done
      }
    }
  }
}

// Precision conversions: two elements per thread and access (16-byte FP64
// loads, 8-byte FP32 stores or the reverse), grid-stride, odd tail last.
__global__ void convert_kernel_f64_f32(const double* __restrict__ a, float* __restrict__ b, long long n) {
  const long long n2 = n >> 1;
  const double2* a2 = reinterpret_cast<const double2*>(a);
  float2* b2 = reinterpret_cast<float2*>(b);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2; i += (long long)gridDim.x * blockDim.x) {
    const double2 x = a2[i];
    b2[i] = make_float2((float)x.x, (float)x.y);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) b[n - 1] = (float)a[n - 1];
}
__global__ void convert_kernel_f32_f64(const float* __restrict__ a, double* __restrict__ b, long long n) {
  const long long n2 = n >> 1;
  const float2* a2 = reinterpret_cast<const float2*>(a);
  double2* b2 = reinterpret_cast<double2*>(b);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n2; i += (long long)gridDim.x * blockDim.x) {
    const float2 x = a2[i];
    b2[i] = make_double2((double)x.x, (double)x.y);
  }
  if ((n & 1) && blockIdx.x == 0 && threadIdx.x == 0) b[n - 1] = (double)a[n - 1];
}
__global__ void convert_kernel_f64_bf16(const double* a, __nv_bfloat16* b, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
    b[i] = __double2bfloat16(a[i]);
}

__global__ void fill_messages_kernel(int ndir, const int* dchi, const long long* msg_off, double* msgs, int kind,
                                     int cplx) {
  const int de = blockIdx.x;
  if (de >= ndir) return;
  const int c = dchi[de];
  for (int i = threadIdx.x; i < c * c; i += blockDim.x) {
    const int b = i % c, a = i / c;
    const double x = kind == GBTN_INIT_ONES ? 1.0 / c : (a == b ? 1.0 : 0.0);
    if (cplx) {
      msgs[2 * (msg_off[de] + i)] = x;
      msgs[2 * (msg_off[de] + i) + 1] = 0.0;
    } else {
      msgs[msg_off[de] + i] = x;
    }
  }
}

__global__ void scale_vertices_kernel(int nv, const VDesc* vd, double* fac, double* bra, const double* scale) {
  const int v = blockIdx.x;
  if (v >= nv) return;
  const long long off = vd[v].a_off;
  const int n = vd[v].n;
  const double sk = scale[2 * v], sb = scale[2 * v + 1];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    fac[off + i] *= sk;
    if (bra) bra[off + i] *= sb;
  }
}

// rescale_messages (beliefpropagationcache.jl:121-139): both messages of an
// edge normalised, the sign of their inner product moved onto the first, and
// both scaled by |<m1, m2>|^(-1/2) so the edge scalar is 1.  FP64 is scarce on
// this part and a warp instruction costs its pipe the same for one edge or
// eight, so four lanes take an edge (eight edges per warp): each lane keeps
// its up-to-16 entries of both messages in registers, the three inner
// products are reduced over the four lanes, and the factors -- three
// reciprocal square roots -- are formed once per instruction for all eight
// edges and applied by multiplication.  A warp reads 8 x 4 consecutive FP64
// values per load (32-byte sectors).
__global__ void rescale_messages_kernel(int ne, const int* dchi, const long long* msg_off, double* msgs) {
  const int e = blockIdx.x * (blockDim.x >> 2) + (threadIdx.x >> 2);
  const int l4 = threadIdx.x & 3;
  const bool ok = e < ne;  // lanes past the last edge still take part in the shuffles
  const int c2 = ok ? dchi[2 * e] * dchi[2 * e] : 0;
  double* m1 = msgs + (ok ? msg_off[2 * e] : 0);
  double* m2 = msgs + (ok ? msg_off[2 * e + 1] : 0);
  double a[16], b[16];
  double na2 = 0.0, nb2 = 0.0, ab = 0.0;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int i = l4 + 4 * j;
    a[j] = i < c2 ? m1[i] : 0.0;
    b[j] = i < c2 ? m2[i] : 0.0;
    na2 = fma(a[j], a[j], na2);
    nb2 = fma(b[j], b[j], nb2);
    ab = fma(a[j], b[j], ab);
  }
#pragma unroll
  for (int o = 1; o < 4; o <<= 1) {
    na2 += __shfl_xor_sync(0xffffffffu, na2, o);
    nb2 += __shfl_xor_sync(0xffffffffu, nb2, o);
    ab += __shfl_xor_sync(0xffffffffu, ab, o);
  }
  const double ia = rsqrt(na2), ib = rsqrt(nb2);
  const double n = ab * ia * ib;  // <m1/|m1|, m2/|m2|>
  const double sg = n > 0.0 ? 1.0 : (n < 0.0 ? -1.0 : 0.0);
  const double isf = rsqrt(fabs(n));
  const double ka = sg * isf * ia, kb = isf * ib;
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int i = l4 + 4 * j;
    if (i < c2) {
      m1[i] = ka * a[j];
      m2[i] = kb * b[j];
    }
  }
}

// Complex messages (rescale_messages, beliefpropagationcache.jl:121-139):
// normalise both, n = sum m1 m2 (no conjugation), and when n is real fix the
// sign of m1 (n -> |n|); then multiply both by the principal n^(-1/2).  One
// warp per edge; the complex networks this serves are not bandwidth-bound.
__global__ void rescale_messages_z_kernel(int ne, const int* dchi, const long long* msg_off, zdouble* msgs) {
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= ne) return;
  const int c2 = dchi[2 * e] * dchi[2 * e];
  zdouble* m1 = msgs + msg_off[2 * e];
  zdouble* m2 = msgs + msg_off[2 * e + 1];
  double na2 = 0.0, nb2 = 0.0, pr = 0.0, pi = 0.0;
  for (int i = lane; i < c2; i += 32) {
    const zdouble a = m1[i], b = m2[i];
    na2 += a.re * a.re + a.im * a.im;
    nb2 += b.re * b.re + b.im * b.im;
    pr += a.re * b.re - a.im * b.im;
    pi += a.re * b.im + a.im * b.re;
  }
  na2 = warp_sum(na2);
  nb2 = warp_sum(nb2);
  pr = warp_sum(pr);
  pi = warp_sum(pi);
  const double ia = 1.0 / sqrt(na2), ib = 1.0 / sqrt(nb2);
  double nr = pr * ia * ib, ni = pi * ia * ib;  // n = <m1/|m1|, m2/|m2|>
  double sg = 1.0;
  if (ni == 0.0) {  // isreal(n): m1 *= sign(n), n *= sign(n)
    sg = nr > 0.0 ? 1.0 : (nr < 0.0 ? -1.0 : 0.0);
    nr *= sg;
  }
  // principal square root of n, then its reciprocal: the larger component from
  // sqrt((|n| + |Re n|) / 2), the other as Im n / (2 * it), so that neither
  // cancels (|n| + Re n loses digits when n is near the negative real axis)
  const double mod = sqrt(nr * nr + ni * ni);
  const double h = sqrt(0.5 * (mod + fabs(nr)));
  const double sr = nr >= 0.0 ? h : (h > 0.0 ? fabs(ni) / (2.0 * h) : 0.0);
  const double si = nr >= 0.0 ? (h > 0.0 ? ni / (2.0 * h) : 0.0) : copysign(h, ni);
  const double sm2 = sr * sr + si * si;
  const double fr = sr / sm2, fi = -si / sm2;  // n^(-1/2)
  const zdouble ka(sg * ia * fr, sg * ia * fi), kb(ib * fr, ib * fi);
  for (int i = lane; i < c2; i += 32) {
    const zdouble a = m1[i], b = m2[i];
    m1[i] = zdouble(ka.re * a.re - ka.im * a.im, ka.re * a.im + ka.im * a.re);
    m2[i] = zdouble(kb.re * b.re - kb.im * b.im, kb.re * b.im + kb.im * b.re);
  }
}

__global__ void edge_scalars_kernel(int ne, const int* dchi, const long long* msg_off, const double* msgs, double* out) {
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= ne) return;
  const int c2 = dchi[2 * e] * dchi[2 * e];
  const double* m1 = msgs + msg_off[2 * e];
  const double* m2 = msgs + msg_off[2 * e + 1];
  double s = 0.0;
  for (int i = lane; i < c2; i += 32) s += m1[i] * m2[i];
  s = warp_sum(s);
  if (lane == 0) out[e] = s;
}

// Complex edge scalar sum_i m1[i] m2[i] (the two messages contracted, no
// conjugation -- ITensors contraction), one warp per edge.
__global__ void edge_scalars_z_kernel(int ne, const int* dchi, const long long* msg_off, const zdouble* msgs,
                                      zdouble* out) {
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= ne) return;
  const int c2 = dchi[2 * e] * dchi[2 * e];
  const zdouble* m1 = msgs + msg_off[2 * e];
  const zdouble* m2 = msgs + msg_off[2 * e + 1];
  double re = 0.0, im = 0.0;
  for (int i = lane; i < c2; i += 32) {
    const zdouble a = m1[i], b = m2[i];
    re = fma(a.re, b.re, fma(-a.im, b.im, re));
    im = fma(a.re, b.im, fma(a.im, b.re, im));
  }
  re = warp_sum(re);
  im = warp_sum(im);
  if (lane == 0) out[e] = zdouble(re, im);
}

// Complex logscalar per network: sum_v Log Z_v - sum_e Log z_e with
// principal logs (log|z| + i arg z), Z_v = tr rho_v; -Inf on a zero edge scalar.
__global__ void logscalar_z_kernel(const int* net_v_ptr, const int* net_v, const int* net_e_ptr, const int* net_e,
                                   const long long* rdm_off, const zdouble* rdm, const int* dsite,
                                   const zdouble* edge_sc, double* re, double* im) {
  const int net = blockIdx.x;
  double lre = 0.0, lim = 0.0, zero_e = 0.0;
  for (int i = net_v_ptr[net] + threadIdx.x; i < net_v_ptr[net + 1]; i += blockDim.x) {
    const int v = net_v[i];
    const int d = dsite[v];
    double zr = 0.0, zi = 0.0;
    for (int s = 0; s < d; ++s) {
      const zdouble x = rdm[rdm_off[v] + s + d * s];
      zr += x.re;
      zi += x.im;
    }
    lre += 0.5 * log(zr * zr + zi * zi);
    lim += atan2(zi, zr);
  }
  for (int i = net_e_ptr[net] + threadIdx.x; i < net_e_ptr[net + 1]; i += blockDim.x) {
    const zdouble z = edge_sc[net_e[i]];
    const double a2 = z.re * z.re + z.im * z.im;
    zero_e += a2 == 0.0 ? 1.0 : 0.0;
    lre -= 0.5 * log(a2);
    lim -= atan2(z.im, z.re);
  }
  __shared__ double red[3][32];
  double vals[3] = {lre, lim, zero_e};
  for (int q = 0; q < 3; ++q) {
    const double t = warp_sum(vals[q]);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double tot[3] = {0.0, 0.0, 0.0};
    for (int q = 0; q < 3; ++q)
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) tot[q] += red[q][w];
    re[net] = tot[2] > 0.0 ? -INFINITY : tot[0];
    im[net] = tot[2] > 0.0 ? 0.0 : tot[1];
  }
}

// Real part of <O_v> = sum rho[a, b] O[a, b] / tr rho from complex RDMs, O real.
__global__ void expect1_z_kernel(int nv, const long long* rdm_off, const zdouble* rdm, const int* dsite,
                                 const double* ops, const long long* op_off, double* out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int d = dsite[v];
  const zdouble* r = rdm + rdm_off[v];
  const double* o = ops + (op_off ? op_off[v] : 0);
  double nr = 0.0, ni = 0.0, dr = 0.0, di = 0.0;
  for (int i = 0; i < d * d; ++i) {
    nr += r[i].re * o[i];
    ni += r[i].im * o[i];
  }
  for (int q = 0; q < d; ++q) {
    dr += r[q + d * q].re;
    di += r[q + d * q].im;
  }
  out[v] = (nr * dr + ni * di) / (dr * dr + di * di);
}

// logscalar per network: sum_v log Z_v - sum_e log z_e in FP64, negative
// terms promoted to complex (log|x| + i*pi), -Inf on a zero edge scalar.
__global__ void logscalar_kernel(const int* net_v_ptr, const int* net_v, const int* net_e_ptr, const int* net_e,
                                 const long long* rdm_off, const double* rdm, const int* dsite, const double* edge_sc,
                                 double* re, double* im) {
  const int net = blockIdx.x;
  double lre = 0.0, neg = 0.0, eneg = 0.0, ere = 0.0, zero_e = 0.0;
  for (int i = net_v_ptr[net] + threadIdx.x; i < net_v_ptr[net + 1]; i += blockDim.x) {
    const int v = net_v[i];
    const int d = dsite[v];
    double z = 0.0;
    for (int s = 0; s < d; ++s) z += rdm[rdm_off[v] + s + d * s];
    lre += log(fabs(z));
    neg += z < 0.0 ? 1.0 : 0.0;
  }
  for (int i = net_e_ptr[net] + threadIdx.x; i < net_e_ptr[net + 1]; i += blockDim.x) {
    const double z = edge_sc[net_e[i]];
    ere += log(fabs(z));
    eneg += z < 0.0 ? 1.0 : 0.0;
    zero_e += z == 0.0 ? 1.0 : 0.0;
  }
  __shared__ double red[5][32];
  double vals[5] = {lre, neg, ere, eneg, zero_e};
  for (int q = 0; q < 5; ++q) {
    const double t = warp_sum(vals[q]);
    if ((threadIdx.x & 31) == 0) red[q][threadIdx.x >> 5] = t;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int q = 0; q < 5; ++q) {
      double t = 0.0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[q][w];
      vals[q] = t;
    }
    const double pi = 3.14159265358979323846;
    if (vals[4] > 0.0) {
      re[net] = -INFINITY;
      im[net] = 0.0;
    } else {
      re[net] = vals[0] - vals[2];
      im[net] = pi * (vals[1] - vals[3]);
    }
  }
}

// ---------------------------------------------------------------------------
// Launchers
// ---------------------------------------------------------------------------

// One size class of a vertex list with its team width: 32 (four vertices per
// 128-thread block), 128 or 256 threads per vertex.  T is the arithmetic, S
// the storage.
template <typename T, typename S>
void launch_vertex_class(const WorkList& wl, const VDesc* vd, const S* fac, const S* bra, const S* msg_in, S* msg_out,
                         const long long* msg_off, double* diffs, const int* converged, int normalize, int want_diff,
                         cudaStream_t s) {
  if (wl.count == 0) return;
  const int nbuf = wl.maxdeg <= 4 ? 3 : kNumBufs;
  const int np = padded_len(wl.ncap);
  if (wl.team == 32) {
    const size_t sm = 4 * team_smem_bytes<T>(np, nbuf, bra != nullptr, 32);
    auto kern = bp_vertex_kernel<T, 32, S>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<(wl.count + 3) / 4, 128, sm, s>>>(wl.d_vertices, wl.count, vd, fac, bra, msg_in, msg_out, msg_off, diffs,
                                             converged, normalize, want_diff, wl.ncap, nbuf);
  } else if (wl.team == 128) {
    const size_t sm = team_smem_bytes<T>(np, nbuf, bra != nullptr, 128);
    auto kern = bp_vertex_kernel<T, 128, S>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<wl.count, 128, sm, s>>>(wl.d_vertices, wl.count, vd, fac, bra, msg_in, msg_out, msg_off, diffs, converged,
                                   normalize, want_diff, wl.ncap, nbuf);
  } else {
    const size_t sm = team_smem_bytes<T>(np, nbuf, bra != nullptr, 256);
    auto kern = bp_vertex_kernel<T, 256, S>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<wl.count, 256, sm, s>>>(wl.d_vertices, wl.count, vd, fac, bra, msg_in, msg_out, msg_off, diffs, converged,
                                   normalize, want_diff, wl.ncap, nbuf);
  }
  GBTN_CUDA(cudaGetLastError());
}

template <typename T>
void launch_bp_vertices(const WorkList& wl_all, const VDesc* vd, const T* fac, const T* bra, const T* msg_in,
                        T* msg_out, const long long* msg_off, double* diffs, const int* converged, int normalize,
                        int want_diff, cudaStream_t s) {
  for (int c = 0; c < wl_all.nsubs(); ++c)
    launch_vertex_class<T, T>(wl_all.sub(c), vd, fac, bra, msg_in, msg_out, msg_off, diffs, converged, normalize,
                              want_diff, s);
}

void launch_bp_vertices_df32(const WorkList& wl_all, const VDesc* vd, const double* fac, const double* bra,
                             const double* msg_in, double* msg_out, const long long* msg_off, double* diffs,
                             const int* converged, int normalize, int want_diff, cudaStream_t s) {
  for (int c = 0; c < wl_all.nsubs(); ++c)
    launch_vertex_class<df32, double>(wl_all.sub(c), vd, fac, bra, msg_in, msg_out, msg_off, diffs, converged,
                                      normalize, want_diff, s);
}

template void launch_bp_vertices<double>(const WorkList&, const VDesc*, const double*, const double*, const double*,
                                         double*, const long long*, double*, const int*, int, int, cudaStream_t);
template void launch_bp_vertices<float>(const WorkList&, const VDesc*, const float*, const float*, const float*, float*,
                                        const long long*, double*, const int*, int, int, cudaStream_t);
template void launch_bp_vertices<zdouble>(const WorkList&, const VDesc*, const zdouble*, const zdouble*,
                                          const zdouble*, zdouble*, const long long*, double*, const int*, int, int,
                                          cudaStream_t);
template void launch_bp_vertices<zfloat>(const WorkList&, const VDesc*, const zfloat*, const zfloat*, const zfloat*,
                                         zfloat*, const long long*, double*, const int*, int, int, cudaStream_t);

template <typename T, typename S>
void launch_bp_wave(const WaveJobs& wj, const VDesc* vd, const S* fac, const S* bra, S* msgs, const long long* msg_off,
                    double* pos_diffs, const int* converged, int normalize, int want_diff, cudaStream_t s) {
  if (wj.count == 0) return;
  if (wj.team == 32) {
    const size_t sm = 4 * team_smem_bytes<T>(padded_len(wj.ncap), 3, bra != nullptr, 32);
    auto kern = bp_wave_kernel<T, 32, S>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<(wj.count + 3) / 4, 128, sm, s>>>(wj.d_jobs, wj.count, vd, fac, bra, msgs, msg_off, pos_diffs, converged,
                                              normalize, want_diff, wj.ncap);
  } else {
    const size_t sm = team_smem_bytes<T>(padded_len(wj.ncap), 3, bra != nullptr, 256);
    auto kern = bp_wave_kernel<T, 256, S>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<wj.count, 256, sm, s>>>(wj.d_jobs, wj.count, vd, fac, bra, msgs, msg_off, pos_diffs, converged, normalize,
                                   want_diff, wj.ncap);
  }
  GBTN_CUDA(cudaGetLastError());
}

void launch_bp_wave_any(int arith, const WaveJobs& wj, const VDesc* vd, const void* fac, const void* bra, void* msgs,
                        const long long* msg_off, double* pos_diffs, const int* converged, int normalize,
                        int want_diff, cudaStream_t s) {
  switch (arith) {
    case kArithF64:
      launch_bp_wave<double, double>(wj, vd, static_cast<const double*>(fac), static_cast<const double*>(bra),
                                     static_cast<double*>(msgs), msg_off, pos_diffs, converged, normalize, want_diff, s);
      break;
    case kArithF32:
      launch_bp_wave<float, float>(wj, vd, static_cast<const float*>(fac), static_cast<const float*>(bra),
                                   static_cast<float*>(msgs), msg_off, pos_diffs, converged, normalize, want_diff, s);
      break;
    case kArithDF32:
      launch_bp_wave<df32, double>(wj, vd, static_cast<const double*>(fac), static_cast<const double*>(bra),
                                   static_cast<double*>(msgs), msg_off, pos_diffs, converged, normalize, want_diff, s);
      break;
    case kArithZ64:
      launch_bp_wave<zdouble, zdouble>(wj, vd, static_cast<const zdouble*>(fac), static_cast<const zdouble*>(bra),
                                       static_cast<zdouble*>(msgs), msg_off, pos_diffs, converged, normalize,
                                       want_diff, s);
      break;
    case kArithZ32:
      launch_bp_wave<zfloat, zfloat>(wj, vd, static_cast<const zfloat*>(fac), static_cast<const zfloat*>(bra),
                                     static_cast<zfloat*>(msgs), msg_off, pos_diffs, converged, normalize, want_diff,
                                     s);
      break;
    default:
      throw std::logic_error("wave kernel: unknown arithmetic");
  }
}

void launch_reduce_diffs(int n_networks, const int* net_de_ptr, const int* net_de, const double* diffs, double tol,
                         int* converged, int* iters, double* mean_diff, cudaStream_t s, int stall, double* best,
                         int* since, int* n_conv) {
  reduce_diffs_kernel<<<n_networks, 256, 0, s>>>(net_de_ptr, net_de, diffs, tol, converged, iters, mean_diff, stall,
                                                 best, since, n_conv);
  GBTN_CUDA(cudaGetLastError());
}

template <typename T>
void launch_updated_message(const VDesc* vd, int v, int leg, const T* fac, const T* bra, const T* msgs,
                            const long long* msg_off, T* out, int ncap, cudaStream_t s) {
  const size_t sm = team_smem_bytes<T>(padded_len(ncap), 3, bra != nullptr, 256);
  GBTN_CUDA(cudaFuncSetAttribute(updated_message_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  updated_message_kernel<T><<<1, 256, sm, s>>>(vd, v, leg, fac, bra, msgs, msg_off, out, ncap);
  GBTN_CUDA(cudaGetLastError());
}
template void launch_updated_message<double>(const VDesc*, int, int, const double*, const double*, const double*,
                                             const long long*, double*, int, cudaStream_t);
template void launch_updated_message<zdouble>(const VDesc*, int, int, const zdouble*, const zdouble*, const zdouble*,
                                              const long long*, zdouble*, int, cudaStream_t);

template <typename T>
void launch_vertex_rdms(const WorkList& wl, const VDesc* vd, const T* fac, const T* bra, const T* msgs,
                        const long long* msg_off, const long long* rdm_off, T* rdm, cudaStream_t s) {
  if (wl.count == 0) return;
  if (wl.team == 32) {
    const size_t sm = 4 * team_smem_bytes<T>(padded_len(wl.ncap), 3, bra != nullptr, 32);
    auto kern = vertex_rdm_kernel<T, 32>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<(wl.count + 3) / 4, 128, sm, s>>>(wl.d_vertices, wl.count, vd, fac, bra, msgs, msg_off, rdm_off, rdm,
                                              wl.ncap);
  } else {
    const size_t sm = team_smem_bytes<T>(padded_len(wl.ncap), 3, bra != nullptr, 256);
    auto kern = vertex_rdm_kernel<T, 256>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<wl.count, 256, sm, s>>>(wl.d_vertices, wl.count, vd, fac, bra, msgs, msg_off, rdm_off, rdm, wl.ncap);
  }
  GBTN_CUDA(cudaGetLastError());
}
template void launch_vertex_rdms<double>(const WorkList&, const VDesc*, const double*, const double*, const double*,
                                         const long long*, const long long*, double*, cudaStream_t);

void launch_vertex_rdms_df32(const WorkList& wl, const VDesc* vd, const double* fac, const double* bra,
                             const double* msgs, const long long* msg_off, const long long* rdm_off, double* rdm,
                             cudaStream_t s) {
  if (wl.count == 0) return;
  if (wl.team == 32) {
    const size_t sm = 4 * team_smem_bytes<df32>(padded_len(wl.ncap), 3, bra != nullptr, 32);
    auto kern = vertex_rdm_kernel<df32, 32, double>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<(wl.count + 3) / 4, 128, sm, s>>>(wl.d_vertices, wl.count, vd, fac, bra, msgs, msg_off, rdm_off, rdm,
                                              wl.ncap);
  } else {
    const size_t sm = team_smem_bytes<df32>(padded_len(wl.ncap), 3, bra != nullptr, 256);
    auto kern = vertex_rdm_kernel<df32, 256, double>;
    GBTN_CUDA(cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
    kern<<<wl.count, 256, sm, s>>>(wl.d_vertices, wl.count, vd, fac, bra, msgs, msg_off, rdm_off, rdm, wl.ncap);
  }
  GBTN_CUDA(cudaGetLastError());
}
template void launch_vertex_rdms<zdouble>(const WorkList&, const VDesc*, const zdouble*, const zdouble*,
                                          const zdouble*, const long long*, const long long*, zdouble*, cudaStream_t);

void launch_edge_scalars_z(int ne, const int* dchi, const long long* msg_off, const zdouble* msgs, zdouble* out,
                           cudaStream_t s) {
  if (ne == 0) return;
  edge_scalars_z_kernel<<<(ne + 7) / 8, 256, 0, s>>>(ne, dchi, msg_off, msgs, out);
  GBTN_CUDA(cudaGetLastError());
}

void launch_logscalar_z(int n_networks, const int* net_v_ptr, const int* net_v, const int* net_e_ptr,
                        const int* net_e, const long long* rdm_off, const zdouble* rdm, const int* dsite,
                        const zdouble* edge_sc, double* re, double* im, cudaStream_t s) {
  logscalar_z_kernel<<<n_networks, 256, 0, s>>>(net_v_ptr, net_v, net_e_ptr, net_e, rdm_off, rdm, dsite, edge_sc,
                                                re, im);
  GBTN_CUDA(cudaGetLastError());
}

void launch_expect1_z(int nv, const long long* rdm_off, const zdouble* rdm, const int* dsite, const double* ops,
                      const long long* op_off, double* out, cudaStream_t s) {
  if (nv == 0) return;
  expect1_z_kernel<<<(nv + 127) / 128, 128, 0, s>>>(nv, rdm_off, rdm, dsite, ops, op_off, out);
  GBTN_CUDA(cudaGetLastError());
}

template <typename T>
void launch_edge_halves(const int* jobs, int njobs, int ncap, int maxdeg, const VDesc* vd, const T* fac, const T* bra,
                        const T* msgs, const long long* msg_off, T* halves, const long long* half_off, cudaStream_t s) {
  (void)maxdeg;
  if (njobs == 0) return;
  const size_t sm = team_smem_bytes<T>(padded_len(ncap), 3, bra != nullptr, 256);
  GBTN_CUDA(cudaFuncSetAttribute(edge_half_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  edge_half_kernel<T><<<njobs, 256, sm, s>>>(reinterpret_cast<const int2*>(jobs), njobs, vd, fac, bra, msgs, msg_off,
                                             halves, half_off, ncap);
  GBTN_CUDA(cudaGetLastError());
}
template void launch_edge_halves<double>(const int*, int, int, int, const VDesc*, const double*, const double*,
                                         const double*, const long long*, double*, const long long*, cudaStream_t);
template void launch_edge_halves<zdouble>(const int*, int, int, int, const VDesc*, const zdouble*, const zdouble*,
                                          const zdouble*, const long long*, zdouble*, const long long*, cudaStream_t);

static int grid_for(long long n) {
  long long b = (n + 255) / 256;
  if (b > 152 * 16) b = 152 * 16;
  return (int)(b < 1 ? 1 : b);
}

void launch_convert_f64_to_f32(const double* a, float* b, long long n, cudaStream_t s) {
  convert_kernel_f64_f32<<<grid_for(n), 256, 0, s>>>(a, b, n);
  GBTN_CUDA(cudaGetLastError());
}
void launch_convert_f32_to_f64(const float* a, double* b, long long n, cudaStream_t s) {
  convert_kernel_f32_f64<<<grid_for(n), 256, 0, s>>>(a, b, n);
  GBTN_CUDA(cudaGetLastError());
}
void launch_convert_f64_to_bf16(const double* a, __nv_bfloat16* b, long long n, cudaStream_t s) {
  convert_kernel_f64_bf16<<<grid_for(n), 256, 0, s>>>(a, b, n);
  GBTN_CUDA(cudaGetLastError());
}
void launch_fill_messages(int ndir, const int* dchi, const long long* msg_off, double* msgs, int kind, cudaStream_t s,
                          int cplx) {
  if (ndir == 0) return;
  fill_messages_kernel<<<ndir, 64, 0, s>>>(ndir, dchi, msg_off, msgs, kind, cplx);
  GBTN_CUDA(cudaGetLastError());
}
void launch_scale_vertices(int nv, const VDesc* vd, double* fac, double* bra, const double* scale, cudaStream_t s) {
  if (nv == 0) return;
  scale_vertices_kernel<<<nv, 256, 0, s>>>(nv, vd, fac, bra, scale);
  GBTN_CUDA(cudaGetLastError());
}
void launch_rescale_messages_z(int ne, const int* dchi, const long long* msg_off, zdouble* msgs, cudaStream_t s) {
  rescale_messages_z_kernel<<<(ne + 7) / 8, 256, 0, s>>>(ne, dchi, msg_off, msgs);
  GBTN_CUDA(cudaGetLastError());
}

// rescale_messages for bond dimensions above 8: one warp per edge, strided
// over the chi^2 entries (the same factors as rescale_messages_kernel).
__global__ void rescale_messages_wide_kernel(int ne, const int* dchi, const long long* msg_off, double* msgs) {
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= ne) return;
  const int c2 = dchi[2 * e] * dchi[2 * e];
  double* m1 = msgs + msg_off[2 * e];
  double* m2 = msgs + msg_off[2 * e + 1];
  double na2 = 0.0, nb2 = 0.0, ab = 0.0;
  for (int i = lane; i < c2; i += 32) {
    const double a = m1[i], b = m2[i];
    na2 = fma(a, a, na2);
    nb2 = fma(b, b, nb2);
    ab = fma(a, b, ab);
  }
  na2 = warp_sum(na2);
  nb2 = warp_sum(nb2);
  ab = warp_sum(ab);
  const double ia = rsqrt(na2), ib = rsqrt(nb2);
  const double n = ab * ia * ib;
  const double sg = n > 0.0 ? 1.0 : (n < 0.0 ? -1.0 : 0.0);
  const double isf = rsqrt(fabs(n));
  const double ka = sg * isf * ia, kb = isf * ib;
  for (int i = lane; i < c2; i += 32) {
    m1[i] *= ka;
    m2[i] *= kb;
  }
}

void launch_rescale_messages(int ne, const int* dchi, const long long* msg_off, double* msgs, cudaStream_t s,
                             int max_chi) {
  if (ne == 0) return;
  if (max_chi <= 8)
    rescale_messages_kernel<<<(ne + 63) / 64, 256, 0, s>>>(ne, dchi, msg_off, msgs);  // 4 lanes per edge
  else
    rescale_messages_wide_kernel<<<(ne + 7) / 8, 256, 0, s>>>(ne, dchi, msg_off, msgs);
  GBTN_CUDA(cudaGetLastError());
}
void launch_edge_scalars(int ne, const int* dchi, const long long* msg_off, const double* msgs, double* out,
                         cudaStream_t s) {
  if (ne == 0) return;
  edge_scalars_kernel<<<(ne + 7) / 8, 256, 0, s>>>(ne, dchi, msg_off, msgs, out);
  GBTN_CUDA(cudaGetLastError());
}
void launch_logscalar(int n_networks, const int* net_v_ptr, const int* net_v, const int* net_e_ptr, const int* net_e,
                      const long long* rdm_off, const double* rdm, const int* dsite, const double* edge_sc, double* re,
                      double* im, cudaStream_t s) {
  logscalar_kernel<<<n_networks, 256, 0, s>>>(net_v_ptr, net_v, net_e_ptr, net_e, rdm_off, rdm, dsite, edge_sc, re, im);
  GBTN_CUDA(cudaGetLastError());
}

}  // namespace gbtn
