// Charge-conserving (QN, U(1)-graded) block-sparse networks: plan, block
// bookkeeping and the kernels that add the blocks' message shares.
//
// ITensors' QN tensors (conserve_qns = true) are block-sparse: every index is
// a list of sectors of one charge, and a tensor is nonzero only in the blocks
// whose charges balance its flux.  BP on such a network (the QN-graded loopy
// case of test/test_belief_propagation.jl:103-116) keeps every message
// block-diagonal in the link sectors: identity messages are, and a message
// built from block-diagonal messages and flux-balanced tensors is again.  So
// the plan stores the nonzero blocks of the tensors and the diagonal sector
// blocks of the messages, and an update is a sum over blocks: the share of a
// block B in the outgoing message on leg p (its sector sigma_p there) is the
// dense update of B alone, with the sector blocks of B's incoming messages,
// because every absorbed message keeps each leg of B in its sector and the
// bra block that closes B has B's own sectors (qn_block_kernel, bp_kernels.cu).
// qn_finalize_kernel adds the shares of all blocks with the same outgoing
// sector, in a fixed order, normalises the whole message in FP64 and records
// message_diff (abstractbeliefpropagationcache.jl:32-36, 225-239).
#include <algorithm>
#include <cmath>
#include <memory>
#include <numeric>
#include <string>
#include <vector>

#include "bp_device.cuh"

namespace gbtn {
cudaStream_t ctx_stream(gbtn_ctx* c);
void set_ctx_error(gbtn_ctx* c, const char* msg);
}  // namespace gbtn

using namespace gbtn;

namespace {

constexpr int kBlockFields = 2 + kMaxDeg;  // vertex, site sector, leg sectors
constexpr int kQnSmallN = 1024;            // blocks up to this size run one per warp
constexpr int kQnStallSweeps = 3;          // noise-floor test of the FP32 phase, as for dense plans

template <typename T>
struct QBuf {
  T* p = nullptr;
  size_t n = 0;
  QBuf() = default;
  QBuf(const QBuf&) = delete;
  QBuf& operator=(const QBuf&) = delete;
  ~QBuf() {
    if (p) cudaFree(p);
  }
  void alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    if (count) GBTN_CUDA(cudaMalloc(&p, count * sizeof(T)));
  }
  void upload(const std::vector<T>& h, cudaStream_t s) {
    alloc(std::max<size_t>(h.size(), 1));
    if (!h.empty()) GBTN_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

// One warp per directed edge: every sector block of the message is the sum of
// the shares of the blocks with that outgoing sector (slot lists in order);
// the message is normalised over all its sectors in FP64 and compared with
// the old one (message_diff).
// de_list / pos_list (may be NULL: job j is directed edge j, diff slot j)
// select the messages of one wave of the sequential schedule, which finalises
// them in place (msg_old == msg_out: each entry is read before it is written,
// by the same lane) and records each diff at its sequence position.
// S is the storage of shares and messages (FP64, or FP32 for the FP32 sweeps):
// the sums, norms and diff are formed in FP64 from the stored values.
template <typename S>
__global__ void qn_finalize_kernel(int ndir, const int* __restrict__ vm_ptr, const int* __restrict__ vm_dim,
                                   const long long* __restrict__ sec_off, const int* __restrict__ slot_ptr,
                                   const int* __restrict__ slots, const long long* __restrict__ part_off,
                                   const S* __restrict__ partial, const S* msg_old, S* msg_out, double* diffs,
                                   int normalize, int want_diff, const int* __restrict__ de_list,
                                   const int* __restrict__ pos_list) {
  const int job = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (job >= ndir) return;
  const int de = de_list ? de_list[job] : job;
  const int pos = pos_list ? pos_list[job] : de;
  double nr2 = 0.0, dot = 0.0, nb = 0.0;
  for (int vm = vm_ptr[de]; vm < vm_ptr[de + 1]; ++vm) {
    const int c2 = vm_dim[vm] * vm_dim[vm];
    const long long off = sec_off[vm];
    for (int i = lane; i < c2; i += 32) {
      double acc = 0.0;
      for (int q = slot_ptr[vm]; q < slot_ptr[vm + 1]; ++q) acc += (double)partial[part_off[slots[q]] + i];
      const S sv = (S)acc;
      const double s = (double)sv, o = (double)msg_old[off + i];
      nr2 = fma(s, s, nr2);
      dot = fma(o, s, dot);
      nb = fma(o, o, nb);
      msg_out[off + i] = sv;
    }
  }
  nr2 = warp_sum(nr2);
  dot = warp_sum(dot);
  nb = warp_sum(nb);
  const double sc = (normalize && nr2 > 0.0) ? 1.0 / sqrt(nr2) : 1.0;
  __syncwarp();
  for (int vm = vm_ptr[de]; vm < vm_ptr[de + 1]; ++vm) {
    const int c2 = vm_dim[vm] * vm_dim[vm];
    const long long off = sec_off[vm];
    for (int i = lane; i < c2; i += 32) msg_out[off + i] = (S)((double)msg_out[off + i] * sc);
  }
  if (want_diff && lane == 0) diffs[pos] = 1.0 - (dot * dot) / (nr2 * nb);
}

// One thread block per vertex: the dense rho_v (d x d) from the shares of its
// blocks, each in the diagonal block of its site sector.
__global__ void qn_rdm_kernel(const int* __restrict__ vb_ptr, const int* __restrict__ vblocks,
                              const int* __restrict__ blk_site_off, const int* __restrict__ blk_ds,
                              const long long* __restrict__ part_off, int rdm_slot0, const double* __restrict__ partial,
                              const long long* __restrict__ rdm_off, const int* __restrict__ dsite, double* rdm) {
  const int v = blockIdx.x;
  const int d = dsite[v];
  double* r = rdm + rdm_off[v];
  for (int i = threadIdx.x; i < d * d; i += blockDim.x) r[i] = 0.0;
  __syncthreads();
  for (int q = vb_ptr[v]; q < vb_ptr[v + 1]; ++q) {
    const int b = vblocks[q];
    const int ds = blk_ds[b], o = blk_site_off[b];
    const double* p = partial + part_off[rdm_slot0 + b];
    for (int i = threadIdx.x; i < ds * ds; i += blockDim.x) r[(o + i % ds) + d * (o + i / ds)] += p[i];
    __syncthreads();
  }
}

// One warp per edge: <m_e, m_ebar> over the sector blocks (the dense
// messages' off-diagonal blocks are zero).
__global__ void qn_edge_scalars_kernel(int ne, const long long* __restrict__ de_off, const int* __restrict__ de_len,
                                       const double* __restrict__ msgs, double* out) {
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= ne) return;
  const double* a = msgs + de_off[2 * e];
  const double* b = msgs + de_off[2 * e + 1];
  double s = 0.0;
  for (int i = lane; i < de_len[2 * e]; i += 32) s = fma(a[i], b[i], s);
  s = warp_sum(s);
  if (lane == 0) out[e] = s;
}

__global__ void qn_identity_kernel(int nvm, const int* __restrict__ vm_dim, const long long* __restrict__ sec_off,
                                   double* msgs) {
  const int vm = blockIdx.x;
  if (vm >= nvm) return;
  const int c = vm_dim[vm];
  for (int i = threadIdx.x; i < c * c; i += blockDim.x) msgs[sec_off[vm] + i] = (i % c == i / c) ? 1.0 : 0.0;
}

void require(bool c, const std::string& m) {
  if (!c) throw InvalidArg(m);
}

}  // namespace

struct gbtn_qn_plan {
  gbtn_ctx* ctx = nullptr;
  int nv = 0, ne = 0, nblocks = 0, nvm = 0;
  long long n_blk = 0, n_msg = 0, n_part = 0, n_rdm = 0;
  std::vector<int> blk_fields;        // nblocks x kBlockFields
  std::vector<long long> blk_off;     // first element of every block
  std::vector<int> dsite;
  WorkList small, large;
  QBuf<int> d_small, d_large;
  QBuf<VDesc> d_bd;
  QBuf<double> d_blocks, d_msg[2], d_partial, d_diffs, d_mean, d_rdm, d_edge_sc, d_re, d_im;
  QBuf<long long> d_sec_off, d_part_off, d_rdm_off, d_de_off;
  QBuf<int> d_vm_ptr, d_vm_dim, d_slot_ptr, d_slots, d_vb_ptr, d_vblocks, d_blk_site_off, d_blk_ds, d_dsite, d_de_len;
  QBuf<int> d_conv, d_iters, d_net_de_ptr, d_net_de, d_net_v_ptr, d_net_v, d_net_e_ptr, d_net_e, d_nconv;
  int cur = 0;
  // the graph (sequential schedule) and the waves of the last edge sequence
  std::vector<int> eu, ev, leg_ptr, leg_edge, vblocks_ptr, vblocks_flat;
  std::vector<VDesc> bd_host;
  std::vector<int> seq_cached;
  std::vector<WorkList> wave_small, wave_large;
  std::vector<int> wave_job_ptr;
  QBuf<int> d_wave_blocks, d_wave_de, d_wave_pos, d_seq_ptr, d_seq_pos;
  // FP32 copies for the FP32 sweeps (made on first use, blocks refreshed per
  // run), the noise-floor state of the reduced-precision phases, and the
  // sweeps each phase of the last run took (0 BF16, 1 FP32, 2 refinement, 3 FP64)
  QBuf<float> d_blocks32, d_msg32[2], d_partial32;
  QBuf<double> d_best;
  QBuf<int> d_since;
  int phase_sweeps[4] = {0, 0, 0, 0};
};

namespace {

#define QN_TRY try {
#define QN_CATCH(CTX)                                          \
  }                                                            \
  catch (const InvalidArg& e) {                                \
    if (CTX) set_ctx_error(CTX, e.what());                     \
    return GBTN_ERR_INVALID;                                   \
  }                                                            \
  catch (const Unsupported& e) {                               \
    if (CTX) set_ctx_error(CTX, e.what());                     \
    return GBTN_ERR_UNSUPPORTED;                               \
  }                                                            \
  catch (const CudaError& e) {                                 \
    if (CTX) set_ctx_error(CTX, e.what());                     \
    return GBTN_ERR_CUDA;                                      \
  }                                                            \
  catch (const std::bad_alloc&) {                              \
    if (CTX) set_ctx_error(CTX, "host allocation failed");     \
    return GBTN_ERR_NOMEM;                                     \
  }                                                            \
  catch (const std::exception& e) {                            \
    if (CTX) set_ctx_error(CTX, e.what());                     \
    return GBTN_ERR_INVALID;                                   \
  }                                                            \
  return GBTN_OK;

size_t block_smem(int n, int k, int team) {
  const int nbuf = k <= 4 ? 3 : kNumBufs;
  return team_smem_bytes<double>(padded_len(n), nbuf, false, team) * (team == 32 ? 4 : 1);
}

WorkList make_qn_list(gbtn_qn_plan* P, const std::vector<VDesc>& bd, const std::vector<int>& ids, int team,
                      QBuf<int>& store) {
  WorkList w;
  w.team = team;
  w.count = (int)ids.size();
  for (int b : ids) {
    w.ncap = std::max(w.ncap, bd[b].n);
    w.maxdeg = std::max(w.maxdeg, bd[b].k);
  }
  store.upload(ids, P->ctx ? ctx_stream(P->ctx) : nullptr);
  w.d_vertices = store.p;
  return w;
}

void copy_h(gbtn_qn_plan* P, void* dst, const void* src, size_t bytes, int mem, bool to_device) {
  cudaStream_t s = ctx_stream(P->ctx);
  const cudaMemcpyKind kind = mem == GBTN_DEVICE ? cudaMemcpyDeviceToDevice
                                                 : (to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost);
  GBTN_CUDA(cudaMemcpyAsync(dst, src, bytes, kind, s));
  GBTN_CUDA(cudaStreamSynchronize(s));
}

// rho_v of every vertex into d_rdm (dense, FP64).
void qn_rdms(gbtn_qn_plan* P) {
  cudaStream_t s = ctx_stream(P->ctx);
  for (const WorkList* wl : {&P->small, &P->large})
    launch_qn_blocks(*wl, P->d_bd.p, P->d_blocks.p, P->d_msg[P->cur].p, P->d_sec_off.p, P->d_partial.p,
                     P->d_part_off.p, 1, s);
  qn_rdm_kernel<<<P->nv, 128, 0, s>>>(P->d_vb_ptr.p, P->d_vblocks.p, P->d_blk_site_off.p, P->d_blk_ds.p,
                                      P->d_part_off.p, P->nblocks * kMaxDeg, P->d_partial.p, P->d_rdm_off.p,
                                      P->d_dsite.p, P->d_rdm.p);
  GBTN_CUDA(cudaGetLastError());
}

// Cut an edge sequence into waves (as the dense plan does): message j goes to
// the first wave after every earlier message it depends on -- the last writer
// of each message it reads (the incoming messages of its source vertex except
// the one from its target), the readers of its own message since that
// message's last write, and its last writer.  A wave runs the block kernel on
// the blocks of its source vertices and finalises its messages in place.
void build_qn_waves(gbtn_qn_plan* P, const int32_t* seq, int len) {
  std::vector<int> key(seq, seq + len);
  if (key == P->seq_cached && !P->wave_job_ptr.empty()) return;
  const int ndir = 2 * P->ne;
  std::vector<int> last_write(ndir, -1), last_read(ndir, -1), level(len, 0);
  int nlev = 0;
  auto src_of = [&](int de) { return (de & 1) ? P->ev[de >> 1] : P->eu[de >> 1]; };
  for (int j = 0; j < len; ++j) {
    const int de = seq[j];
    require(de >= 0 && de < ndir, "edge_sequence entry out of range");
    const int v = src_of(de), e = de >> 1;
    int lv = 0;
    std::vector<int> reads;
    for (int q = P->leg_ptr[v]; q < P->leg_ptr[v + 1]; ++q) {
      const int f = P->leg_edge[q];
      if (f == e) continue;
      const int din = 2 * f + (P->eu[f] == v ? 1 : 0);  // the message into v along f
      reads.push_back(din);
      lv = std::max(lv, last_write[din] + 1);
    }
    lv = std::max(lv, last_read[de] + 1);
    lv = std::max(lv, last_write[de] + 1);
    level[j] = lv;
    nlev = std::max(nlev, lv + 1);
    last_write[de] = lv;
    for (int din : reads) last_read[din] = std::max(last_read[din], lv);
  }
  std::vector<std::vector<int>> jobs(nlev);
  for (int j = 0; j < len; ++j) jobs[level[j]].push_back(j);
  std::vector<int> blocks_flat, de_flat, pos_flat;
  std::vector<std::pair<int, int>> ranges_small, ranges_large;  // (offset, count) into blocks_flat
  P->wave_job_ptr.assign(1, 0);
  std::vector<int> seen(P->nv, -1);
  for (int l = 0; l < nlev; ++l) {
    std::vector<int> sm, lg;
    for (int j : jobs[l]) {
      de_flat.push_back(seq[j]);
      pos_flat.push_back(j);
      const int v = src_of(seq[j]);
      if (seen[v] == l) continue;
      seen[v] = l;
      for (int q = P->vblocks_ptr[v]; q < P->vblocks_ptr[v + 1]; ++q) {
        const int b = P->vblocks_flat[q];
        (P->bd_host[b].n <= kQnSmallN ? sm : lg).push_back(b);
      }
    }
    P->wave_job_ptr.push_back((int)de_flat.size());
    ranges_small.push_back({(int)blocks_flat.size(), (int)sm.size()});
    blocks_flat.insert(blocks_flat.end(), sm.begin(), sm.end());
    ranges_large.push_back({(int)blocks_flat.size(), (int)lg.size()});
    blocks_flat.insert(blocks_flat.end(), lg.begin(), lg.end());
  }
  cudaStream_t s = ctx_stream(P->ctx);
  if (blocks_flat.empty()) blocks_flat.push_back(0);
  if (de_flat.empty()) {
    de_flat.push_back(0);
    pos_flat.push_back(0);
  }
  P->d_wave_blocks.upload(blocks_flat, s);
  P->d_wave_de.upload(de_flat, s);
  P->d_wave_pos.upload(pos_flat, s);
  std::vector<int> pos_all(std::max(len, 1));
  std::iota(pos_all.begin(), pos_all.end(), 0);
  P->d_seq_pos.upload(pos_all, s);
  P->d_seq_ptr.upload(std::vector<int>{0, len}, s);
  P->d_diffs.alloc(std::max({2 * P->ne, len, 1}));
  P->wave_small.clear();
  P->wave_large.clear();
  for (int l = 0; l < nlev; ++l) {
    for (int which = 0; which < 2; ++which) {
      const auto r = which == 0 ? ranges_small[l] : ranges_large[l];
      WorkList w;
      w.team = which == 0 ? 32 : 256;
      w.count = r.second;
      w.d_vertices = P->d_wave_blocks.p + r.first;
      for (int i = 0; i < r.second; ++i) {
        const VDesc& d = P->bd_host[blocks_flat[r.first + i]];
        w.ncap = std::max(w.ncap, d.n);
        w.maxdeg = std::max(w.maxdeg, d.k);
      }
      (which == 0 ? P->wave_small : P->wave_large).push_back(w);
    }
  }
  P->seq_cached = key;
}

// One sweep: the block kernel (blocks(worklist, messages in, shares)) on every
// block, then the finalize.  Parallel: all messages from msg_in into msg_out.
// Sequential: wave by wave, each wave finalising its messages in place in
// msg_in (msg_out unused).
template <typename S, typename Blocks>
void qn_sweep(gbtn_qn_plan* P, const Blocks& blocks, S* partial, S* msg_in, S* msg_out, bool seq, int normalize,
              bool want_diff, cudaStream_t s) {
  if (!seq) {
    for (const WorkList* wl : {&P->small, &P->large})
      if (wl->count) blocks(*wl, msg_in, partial);
    const int ndir = 2 * P->ne;
    qn_finalize_kernel<S><<<(ndir + 7) / 8, 256, 0, s>>>(ndir, P->d_vm_ptr.p, P->d_vm_dim.p, P->d_sec_off.p,
                                                         P->d_slot_ptr.p, P->d_slots.p, P->d_part_off.p, partial,
                                                         msg_in, msg_out, P->d_diffs.p, normalize, want_diff ? 1 : 0,
                                                         nullptr, nullptr);
    GBTN_CUDA(cudaGetLastError());
    return;
  }
  for (size_t l = 0; l + 1 < P->wave_job_ptr.size(); ++l) {
    for (const WorkList* wl : {&P->wave_small[l], &P->wave_large[l]})
      if (wl->count) blocks(*wl, msg_in, partial);
    const int j0 = P->wave_job_ptr[l], nj = P->wave_job_ptr[l + 1] - j0;
    qn_finalize_kernel<S><<<(nj + 7) / 8, 256, 0, s>>>(nj, P->d_vm_ptr.p, P->d_vm_dim.p, P->d_sec_off.p,
                                                       P->d_slot_ptr.p, P->d_slots.p, P->d_part_off.p, partial, msg_in,
                                                       msg_in, P->d_diffs.p, normalize, want_diff ? 1 : 0,
                                                       P->d_wave_de.p + j0, P->d_wave_pos.p + j0);
    GBTN_CUDA(cudaGetLastError());
  }
}

// Sweeps of one arithmetic until the mean diff is <= tol (tol < 0: no test),
// the noise floor (stall > 0: the mean diff has not dropped below 0.9x its
// best for `stall` sweeps) or maxiter sweeps; msg[cur] holds the messages and
// cur follows the parallel sweeps' double buffer.  Returns the sweeps run; md
// gets the last mean diff (NAN without a test).
template <typename S, typename Blocks>
int qn_phase(gbtn_qn_plan* P, const Blocks& blocks, S* partial, S* const msg[2], int& cur, bool seq, int maxiter,
             double tol, int normalize, int stall, double* md) {
  cudaStream_t s = ctx_stream(P->ctx);
  const bool test = tol >= 0.0 || stall > 0;
  *md = NAN;
  GBTN_CUDA(cudaMemsetAsync(P->d_conv.p, 0, sizeof(int), s));
  GBTN_CUDA(cudaMemsetAsync(P->d_iters.p, 0, sizeof(int), s));
  for (int it = 1; it <= maxiter; ++it) {
    qn_sweep<S>(P, blocks, partial, msg[cur], msg[cur ^ 1], seq, normalize, test, s);
    if (!seq) cur ^= 1;
    if (test) {
      launch_reduce_diffs(1, seq ? P->d_seq_ptr.p : P->d_net_de_ptr.p, seq ? P->d_seq_pos.p : P->d_net_de.p,
                          P->d_diffs.p, tol, P->d_conv.p, P->d_iters.p, P->d_mean.p, s, stall, P->d_best.p,
                          P->d_since.p);
      int conv = 0;
      GBTN_CUDA(cudaMemcpyAsync(&conv, P->d_conv.p, sizeof(int), cudaMemcpyDeviceToHost, s));
      GBTN_CUDA(cudaMemcpyAsync(md, P->d_mean.p, sizeof(double), cudaMemcpyDeviceToHost, s));
      GBTN_CUDA(cudaStreamSynchronize(s));
      if (conv) return it;
    }
  }
  return maxiter;
}

auto f64_blocks(gbtn_qn_plan* P) {
  return [P](const WorkList& wl, const double* m, double* part) {
    launch_qn_blocks(wl, P->d_bd.p, P->d_blocks.p, m, P->d_sec_off.p, part, P->d_part_off.p, 0, ctx_stream(P->ctx));
  };
}

auto df32_blocks(gbtn_qn_plan* P) {
  return [P](const WorkList& wl, const double* m, double* part) {
    launch_qn_blocks_df32(wl, P->d_bd.p, P->d_blocks.p, m, P->d_sec_off.p, part, P->d_part_off.p,
                          ctx_stream(P->ctx));
  };
}

auto f32_blocks(gbtn_qn_plan* P) {
  return [P](const WorkList& wl, const float* m, float* part) {
    launch_qn_blocks_f32(wl, P->d_bd.p, P->d_blocks32.p, m, P->d_sec_off.p, part, P->d_part_off.p,
                         ctx_stream(P->ctx));
  };
}

// FP32 sweeps from the FP64 messages and back (the blocks rounded to FP32
// afresh, so later changes of the FP64 blocks are seen).
int qn_f32_phase(gbtn_qn_plan* P, bool seq, int maxiter, double tol, int normalize, int stall, double* md) {
  cudaStream_t s = ctx_stream(P->ctx);
  if (!P->d_msg32[0].p) {
    P->d_blocks32.alloc(std::max<long long>(P->n_blk, 1));
    P->d_msg32[0].alloc(std::max<long long>(P->n_msg, 1));
    P->d_msg32[1].alloc(std::max<long long>(P->n_msg, 1));
    P->d_partial32.alloc(std::max<long long>(P->n_part, 1));
  }
  launch_convert_f64_to_f32(P->d_blocks.p, P->d_blocks32.p, P->n_blk, s);
  launch_convert_f64_to_f32(P->d_msg[P->cur].p, P->d_msg32[0].p, P->n_msg, s);
  float* const m32[2] = {P->d_msg32[0].p, P->d_msg32[1].p};
  int c32 = 0;
  const int n = qn_phase<float>(P, f32_blocks(P), P->d_partial32.p, m32, c32, seq, maxiter, tol, normalize, stall, md);
  launch_convert_f32_to_f64(P->d_msg32[c32].p, P->d_msg[P->cur].p, P->n_msg, s);
  return n;
}

}  // namespace

extern "C" {

int gbtn_qn_bp_run_sequential(gbtn_qn_plan* P, const int32_t* edge_sequence, int32_t len, int32_t maxiter,
                              double tol, int32_t* iters, double* mean_diff) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P && (edge_sequence || len == 0), "NULL argument");
  require(maxiter >= 1, "You need to specify a number of iterations for BP!");
  require(len >= 0, "edge_sequence_len must be >= 0");
  for (int& n : P->phase_sweeps) n = 0;
  double md = NAN;
  int it = maxiter;
  if (len > 0) {
    build_qn_waves(P, edge_sequence, len);
    double* const m[2] = {P->d_msg[P->cur].p, P->d_msg[P->cur].p};
    int cur = 0;
    it = qn_phase<double>(P, f64_blocks(P), P->d_partial.p, m, cur, true, maxiter, tol, 1, 0, &md);
    P->phase_sweeps[3] = it;
  }
  GBTN_CUDA(cudaStreamSynchronize(ctx_stream(P->ctx)));
  if (iters) *iters = it;
  if (mean_diff) *mean_diff = tol >= 0.0 && len > 0 ? md : NAN;
  QN_CATCH(C)
}

int gbtn_qn_plan_create(gbtn_ctx* ctx, const gbtn_graph_desc* g, const gbtn_qn_desc* q, gbtn_qn_plan** out) {
  QN_TRY
  require(ctx && g && q && out, "NULL argument");
  *out = nullptr;
  require(g->nv >= 1 && g->ne >= 0, "graph needs nv >= 1 and ne >= 0");
  require(g->site_dim && g->leg_ptr && (g->ne == 0 || (g->edge_u && g->edge_v && g->edge_dim && g->leg_edge)),
          "graph arrays are NULL");
  require(q->edge_sec_ptr && q->site_sec_ptr && q->site_sec_dim && q->site_sec_charge && q->flux &&
              (g->ne == 0 || (q->sec_dim && q->sec_charge)),
          "QN arrays are NULL");
  if (g->complex_values || g->separate_bra) throw Unsupported("QN plans take real tensors with bra = conj(ket)");
  auto P = std::make_unique<gbtn_qn_plan>();
  P->ctx = ctx;
  cudaStream_t s = ctx_stream(ctx);
  const int nv = g->nv, ne = g->ne;
  P->nv = nv;
  P->ne = ne;
  // sectors
  for (int e = 0; e < ne; ++e) {
    require(g->edge_u[e] >= 0 && g->edge_u[e] < nv && g->edge_v[e] >= 0 && g->edge_v[e] < nv &&
                g->edge_u[e] != g->edge_v[e],
            "edge endpoint out of range or self loop");
    require(q->edge_sec_ptr[e + 1] > q->edge_sec_ptr[e], "every link needs at least one sector");
    int tot = 0;
    for (int k = q->edge_sec_ptr[e]; k < q->edge_sec_ptr[e + 1]; ++k) {
      require(q->sec_dim[k] >= 1, "sector dimensions must be >= 1");
      if (q->sec_dim[k] > kMaxChi) throw Unsupported("link sector dimensions must be in 1..8");
      tot += q->sec_dim[k];
    }
    require(tot == g->edge_dim[e], "the sector dimensions of a link must add up to its dimension");
  }
  // block-diagonal messages need the sectors of an index to carry distinct
  // charges (equal-charge sectors would couple); merge such sectors first
  auto distinct = [&](const int32_t* ch, int b, int e_) {
    std::vector<int> c(ch + b, ch + e_);
    std::sort(c.begin(), c.end());
    return std::adjacent_find(c.begin(), c.end()) == c.end();
  };
  for (int e = 0; e < ne; ++e)
    if (!distinct(q->sec_charge, q->edge_sec_ptr[e], q->edge_sec_ptr[e + 1]))
      throw Unsupported("the sectors of a link must carry distinct charges");
  for (int v = 0; v < nv; ++v)
    if (!distinct(q->site_sec_charge, q->site_sec_ptr[v], q->site_sec_ptr[v + 1]))
      throw Unsupported("the sectors of a site index must carry distinct charges");
  P->dsite.assign(g->site_dim, g->site_dim + nv);
  for (int v = 0; v < nv; ++v) {
    require(q->site_sec_ptr[v + 1] > q->site_sec_ptr[v], "every site index needs at least one sector");
    int tot = 0;
    for (int k = q->site_sec_ptr[v]; k < q->site_sec_ptr[v + 1]; ++k) {
      require(q->site_sec_dim[k] >= 1, "sector dimensions must be >= 1");
      if (q->site_sec_dim[k] > kMaxSite) throw Unsupported("site sector dimensions must be in 1..8");
      tot += q->site_sec_dim[k];
    }
    require(tot == g->site_dim[v], "the sector dimensions of a site index must add up to its dimension");
  }
  // virtual message ids: (directed edge, sector)
  std::vector<int> vm_ptr(2 * ne + 1, 0), vm_dim;
  std::vector<long long> sec_off, de_off(2 * (size_t)ne);
  std::vector<int> de_len(2 * (size_t)ne);
  long long off = 0;
  for (int de = 0; de < 2 * ne; ++de) {
    const int e = de / 2;
    de_off[de] = off;
    const long long start = off;
    for (int k = q->edge_sec_ptr[e]; k < q->edge_sec_ptr[e + 1]; ++k) {
      vm_dim.push_back(q->sec_dim[k]);
      sec_off.push_back(off);
      off += (long long)q->sec_dim[k] * q->sec_dim[k];
    }
    de_len[de] = (int)(off - start);
    vm_ptr[de + 1] = (int)vm_dim.size();
  }
  P->n_msg = off;
  P->nvm = (int)vm_dim.size();
  // blocks: every combination of sectors whose charges balance the flux
  std::vector<VDesc> bd;
  std::vector<int> site_off_of_block, ds_of_block;
  std::vector<std::vector<int>> vblocks(nv);
  std::vector<long long> part_off;
  long long boff = 0, poff = 0;
  std::vector<std::vector<int>> out_slots(P->nvm);  // slot lists of every outgoing (de, sector)
  for (int v = 0; v < nv; ++v) {
    const int b0 = g->leg_ptr[v], b1 = g->leg_ptr[v + 1];
    require(b1 >= b0, "leg_ptr must be non-decreasing");
    const int k = b1 - b0;
    if (k > kMaxDeg) throw Unsupported("vertex degree above 8");
    std::vector<int> legs(k), nsec(k + 1), first(k + 1);
    nsec[0] = q->site_sec_ptr[v + 1] - q->site_sec_ptr[v];
    first[0] = q->site_sec_ptr[v];
    for (int p = 0; p < k; ++p) {
      const int e = g->leg_edge[b0 + p];
      require(e >= 0 && e < ne && (g->edge_u[e] == v || g->edge_v[e] == v), "leg_edge names a foreign edge");
      legs[p] = e;
      nsec[p + 1] = q->edge_sec_ptr[e + 1] - q->edge_sec_ptr[e];
      first[p + 1] = q->edge_sec_ptr[e];
    }
    std::vector<int> idx(k + 1, 0);  // odometer: site sector fastest, then leg 0, 1, ...
    while (true) {
      long long charge = q->site_sec_charge[first[0] + idx[0]];
      for (int p = 0; p < k; ++p) {
        const int e = legs[p];
        const int c = q->sec_charge[first[p + 1] + idx[p + 1]];
        charge += g->edge_u[e] == v ? -c : c;
      }
      if (charge == q->flux[v]) {
        const int b = (int)bd.size();
        VDesc d{};
        d.k = k;
        d.d = q->site_sec_dim[first[0] + idx[0]];
        d.a_off = boff;
        long long n = d.d;
        std::vector<int> f(kBlockFields, -1);
        f[0] = v;
        f[1] = idx[0];
        for (int p = 0; p < k; ++p) {
          const int e = legs[p];
          const int sk = idx[p + 1];
          d.chi[p] = q->sec_dim[first[p + 1] + sk];
          d.st[p] = (int)n;
          n *= d.chi[p];
          const int out_de = g->edge_u[e] == v ? 2 * e : 2 * e + 1;
          d.in_de[p] = vm_ptr[out_de ^ 1] + sk;  // incoming (directed edge, sector) message
          d.out_de[p] = b * kMaxDeg + p;          // this block's share slot on leg p
          out_slots[vm_ptr[out_de] + sk].push_back(b * kMaxDeg + p);
          f[2 + p] = sk;
        }
        d.n = (int)n;
        d.net = b;  // rho_v share slot (offset by nblocks * kMaxDeg below)
        const int team = n <= kQnSmallN ? 32 : 256;
        if (block_smem((int)n, k, team) > 227 * 1024) throw Unsupported("a QN block is too large for the block kernel");
        bd.push_back(d);
        P->blk_fields.insert(P->blk_fields.end(), f.begin(), f.end());
        P->blk_off.push_back(boff);
        boff += n;
        int so = 0;
        for (int j = 0; j < idx[0]; ++j) so += q->site_sec_dim[first[0] + j];
        site_off_of_block.push_back(so);
        ds_of_block.push_back(d.d);
        vblocks[v].push_back(b);
      }
      int p = 0;
      while (p <= k && ++idx[p] == nsec[p]) idx[p++] = 0;
      if (p > k) break;
    }
  }
  P->nblocks = (int)bd.size();
  P->n_blk = boff;
  require(P->nblocks > 0, "no block of any tensor balances its flux");
  // share slots: nblocks * kMaxDeg message slots, then nblocks rho slots
  part_off.assign((size_t)P->nblocks * kMaxDeg + P->nblocks, 0);
  for (int b = 0; b < P->nblocks; ++b) {
    for (int p = 0; p < bd[b].k; ++p) {
      part_off[(size_t)b * kMaxDeg + p] = poff;
      poff += (long long)bd[b].chi[p] * bd[b].chi[p];
    }
  }
  for (int b = 0; b < P->nblocks; ++b) {
    part_off[(size_t)P->nblocks * kMaxDeg + b] = poff;
    poff += (long long)bd[b].d * bd[b].d;
    bd[b].net = P->nblocks * kMaxDeg + b;
  }
  P->n_part = poff;
  std::vector<int> slot_ptr(1, 0), slots;
  for (const auto& l : out_slots) {
    slots.insert(slots.end(), l.begin(), l.end());
    slot_ptr.push_back((int)slots.size());
  }
  // work lists by block size
  std::vector<int> sm, lg;
  for (int b = 0; b < P->nblocks; ++b) (bd[b].n <= kQnSmallN ? sm : lg).push_back(b);
  P->small = make_qn_list(P.get(), bd, sm, 32, P->d_small);
  P->large = make_qn_list(P.get(), bd, lg, 256, P->d_large);
  // environments
  std::vector<int> vb_ptr(1, 0), vbl;
  std::vector<long long> rdm_off(nv);
  long long roff = 0;
  for (int v = 0; v < nv; ++v) {
    vbl.insert(vbl.end(), vblocks[v].begin(), vblocks[v].end());
    vb_ptr.push_back((int)vbl.size());
    rdm_off[v] = roff;
    roff += (long long)P->dsite[v] * P->dsite[v];
  }
  P->n_rdm = roff;
  // the graph and the blocks of every vertex, for the sequential schedule
  P->eu.assign(g->edge_u, g->edge_u + ne);
  P->ev.assign(g->edge_v, g->edge_v + ne);
  P->leg_ptr.assign(g->leg_ptr, g->leg_ptr + nv + 1);
  P->leg_edge.assign(g->leg_edge, g->leg_edge + g->leg_ptr[nv]);
  P->vblocks_ptr = vb_ptr;
  P->vblocks_flat = vbl;
  P->bd_host = bd;
  // device arrays
  P->d_bd.upload(bd, s);
  P->d_vm_ptr.upload(vm_ptr, s);
  P->d_vm_dim.upload(vm_dim, s);
  P->d_sec_off.upload(sec_off, s);
  P->d_part_off.upload(part_off, s);
  P->d_slot_ptr.upload(slot_ptr, s);
  P->d_slots.upload(slots, s);
  P->d_vb_ptr.upload(vb_ptr, s);
  P->d_vblocks.upload(vbl, s);
  P->d_blk_site_off.upload(site_off_of_block, s);
  P->d_blk_ds.upload(ds_of_block, s);
  P->d_dsite.upload(P->dsite, s);
  P->d_rdm_off.upload(rdm_off, s);
  P->d_de_off.upload(de_off, s);
  P->d_de_len.upload(de_len, s);
  P->d_blocks.alloc(std::max<long long>(P->n_blk, 1));
  GBTN_CUDA(cudaMemsetAsync(P->d_blocks.p, 0, sizeof(double) * P->d_blocks.n, s));
  P->d_msg[0].alloc(std::max<long long>(P->n_msg, 1));
  P->d_msg[1].alloc(std::max<long long>(P->n_msg, 1));
  P->d_partial.alloc(std::max<long long>(P->n_part, 1));
  P->d_diffs.alloc(std::max(2 * ne, 1));
  P->d_rdm.alloc(std::max<long long>(P->n_rdm, 1));
  P->d_edge_sc.alloc(std::max(ne, 1));
  P->d_re.alloc(1);
  P->d_im.alloc(1);
  P->d_mean.alloc(1);
  P->d_conv.alloc(1);
  P->d_iters.alloc(1);
  P->d_nconv.alloc(1);
  P->d_best.alloc(1);
  P->d_since.alloc(1);
  std::vector<int> all_de(std::max(2 * ne, 1)), all_v(nv), all_e(std::max(ne, 1));
  std::iota(all_de.begin(), all_de.end(), 0);
  std::iota(all_v.begin(), all_v.end(), 0);
  std::iota(all_e.begin(), all_e.end(), 0);
  P->d_net_de_ptr.upload(std::vector<int>{0, 2 * ne}, s);
  P->d_net_de.upload(all_de, s);
  P->d_net_v_ptr.upload(std::vector<int>{0, nv}, s);
  P->d_net_v.upload(all_v, s);
  P->d_net_e_ptr.upload(std::vector<int>{0, ne}, s);
  P->d_net_e.upload(all_e, s);
  if (P->nvm)
    qn_identity_kernel<<<P->nvm, 64, 0, s>>>(P->nvm, P->d_vm_dim.p, P->d_sec_off.p, P->d_msg[0].p);
  GBTN_CUDA(cudaGetLastError());
  GBTN_CUDA(cudaStreamSynchronize(s));
  *out = P.release();
  QN_CATCH(ctx)
}

int gbtn_qn_plan_destroy(gbtn_qn_plan* P) {
  if (!P) return GBTN_OK;
  cudaStreamSynchronize(ctx_stream(P->ctx));
  delete P;
  return GBTN_OK;
}

int gbtn_qn_plan_sizes(const gbtn_qn_plan* P, int32_t* n_blocks, int64_t* n_block_elems, int64_t* n_message) {
  if (!P) return GBTN_ERR_INVALID;
  if (n_blocks) *n_blocks = P->nblocks;
  if (n_block_elems) *n_block_elems = P->n_blk;
  if (n_message) *n_message = P->n_msg;
  return GBTN_OK;
}

int gbtn_qn_blocks(const gbtn_qn_plan* P, int32_t* blocks, int64_t* offsets) {
  if (!P) return GBTN_ERR_INVALID;
  if (blocks) std::copy(P->blk_fields.begin(), P->blk_fields.end(), blocks);
  if (offsets) std::copy(P->blk_off.begin(), P->blk_off.end(), offsets);
  return GBTN_OK;
}

int gbtn_qn_set_blocks(gbtn_qn_plan* P, const double* data, int mem) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P && data, "NULL argument");
  copy_h(P, P->d_blocks.p, data, sizeof(double) * P->n_blk, mem, true);
  QN_CATCH(C)
}

int gbtn_qn_init_messages(gbtn_qn_plan* P) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P, "NULL plan");
  cudaStream_t s = ctx_stream(P->ctx);
  if (P->nvm) qn_identity_kernel<<<P->nvm, 64, 0, s>>>(P->nvm, P->d_vm_dim.p, P->d_sec_off.p, P->d_msg[P->cur].p);
  GBTN_CUDA(cudaGetLastError());
  QN_CATCH(C)
}

int gbtn_qn_set_messages(gbtn_qn_plan* P, const double* m, int mem) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P && m, "NULL argument");
  copy_h(P, P->d_msg[P->cur].p, m, sizeof(double) * P->n_msg, mem, true);
  QN_CATCH(C)
}

int gbtn_qn_get_messages(gbtn_qn_plan* P, double* m, int mem) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P && m, "NULL argument");
  copy_h(P, m, P->d_msg[P->cur].p, sizeof(double) * P->n_msg, mem, false);
  QN_CATCH(C)
}

int gbtn_qn_bp_run(gbtn_qn_plan* P, int32_t maxiter, double tol, int32_t* iters, double* mean_diff) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P, "NULL plan");
  require(maxiter >= 1, "You need to specify a number of iterations for BP!");
  for (int& n : P->phase_sweeps) n = 0;
  double md = NAN;
  int it = 1;
  if (P->ne > 0) {
    double* const m[2] = {P->d_msg[0].p, P->d_msg[1].p};
    it = qn_phase<double>(P, f64_blocks(P), P->d_partial.p, m, P->cur, false, maxiter, tol, 1, 0, &md);
    P->phase_sweeps[3] = it;
  }
  GBTN_CUDA(cudaStreamSynchronize(ctx_stream(P->ctx)));
  if (iters) *iters = it;
  if (mean_diff) *mean_diff = tol >= 0.0 ? md : NAN;
  QN_CATCH(C)
}

int gbtn_qn_bp_run_ex(gbtn_qn_plan* P, const gbtn_bp_opts* o, int32_t* iters, double* mean_diff) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P && o, "NULL argument");
  require(o->maxiter >= 1, "You need to specify a number of iterations for BP!");
  require(o->schedule == GBTN_SCHED_PARALLEL || o->schedule == GBTN_SCHED_SEQUENTIAL,
          "block-sparse plans run the parallel or the sequential schedule");
  require(o->precision >= 0 && o->precision <= 4, "unknown precision");
  require(o->refine == GBTN_REFINE_DF32 || o->refine == GBTN_REFINE_F64, "unknown refinement arithmetic");
  require(o->confirm_f64 >= 0, "confirm_f64 must be >= 0");
  if (o->precision == GBTN_BF16) throw Unsupported("block-sparse plans have no tensor-core (BF16) path");
  for (int& n : P->phase_sweeps) n = 0;
  const bool seq = o->schedule == GBTN_SCHED_SEQUENTIAL;
  if (seq) {
    require(o->edge_sequence && o->edge_sequence_len > 0, "SEQUENTIAL needs an edge sequence");
    build_qn_waves(P, o->edge_sequence, o->edge_sequence_len);
  }
  double md = NAN;
  int last = o->maxiter;
  if (P->ne > 0) {
    double* const m[2] = {seq ? P->d_msg[P->cur].p : P->d_msg[0].p, seq ? P->d_msg[P->cur].p : P->d_msg[1].p};
    int seq_cur = 0;
    int& cur = seq ? seq_cur : P->cur;
    auto fp64 = [&](int maxit, int slot) {
      last = qn_phase<double>(P, f64_blocks(P), P->d_partial.p, m, cur, seq, maxit, o->tol, o->normalize, 0, &md);
      P->phase_sweeps[slot] = last;
    };
    auto df32 = [&](int maxit) {
      last = qn_phase<double>(P, df32_blocks(P), P->d_partial.p, m, cur, seq, maxit, o->tol, o->normalize, 0, &md);
      P->phase_sweeps[2] = last;
    };
    if (o->precision == GBTN_F64) {
      fp64(o->maxiter, 3);
    } else if (o->precision == GBTN_DF32) {
      df32(o->maxiter);
    } else if (o->precision == GBTN_F32) {
      last = qn_f32_phase(P, seq, o->maxiter, o->tol, o->normalize, 0, &md);
      P->phase_sweeps[1] = last;
    } else {  // MIXED: FP32 to its tolerance or noise floor, then DF32 (or FP64) to tol
      const double tol32 = o->tol_f32 > 0 ? o->tol_f32 : 1e-13;
      const int it32 = o->maxiter_f32 > 0 ? o->maxiter_f32 : o->maxiter;
      P->phase_sweeps[1] = qn_f32_phase(P, seq, it32, tol32, o->normalize, kQnStallSweeps, &md);
      const int nref = o->refine_f64 > 0 ? std::min(o->refine_f64, o->maxiter) : o->maxiter;
      if (o->refine == GBTN_REFINE_F64) {
        fp64(nref, 2);
      } else {
        df32(nref);
        if (o->confirm_f64 > 0) fp64(std::min(o->confirm_f64, o->maxiter), 3);
      }
    }
  }
  GBTN_CUDA(cudaStreamSynchronize(ctx_stream(P->ctx)));
  if (iters) *iters = last;
  if (mean_diff) *mean_diff = o->tol >= 0.0 && P->ne > 0 ? md : NAN;
  QN_CATCH(C)
}

int gbtn_qn_phase_sweeps(const gbtn_qn_plan* P, int32_t* sweeps) {
  if (!P || !sweeps) return GBTN_ERR_INVALID;
  for (int k = 0; k < 4; ++k) sweeps[k] = P->phase_sweeps[k];
  return GBTN_OK;
}

int gbtn_qn_vertex_rdms(gbtn_qn_plan* P, double* out) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P && out, "NULL argument");
  qn_rdms(P);
  copy_h(P, out, P->d_rdm.p, sizeof(double) * P->n_rdm, GBTN_HOST, false);
  QN_CATCH(C)
}

int gbtn_qn_logscalar(gbtn_qn_plan* P, double* re, double* im) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  QN_TRY
  require(P && re && im, "NULL argument");
  cudaStream_t s = ctx_stream(P->ctx);
  qn_rdms(P);
  if (P->ne)
    qn_edge_scalars_kernel<<<(P->ne + 7) / 8, 256, 0, s>>>(P->ne, P->d_de_off.p, P->d_de_len.p, P->d_msg[P->cur].p,
                                                           P->d_edge_sc.p);
  GBTN_CUDA(cudaGetLastError());
  launch_logscalar(1, P->d_net_v_ptr.p, P->d_net_v.p, P->d_net_e_ptr.p, P->d_net_e.p, P->d_rdm_off.p, P->d_rdm.p,
                   P->d_dsite.p, P->d_edge_sc.p, P->d_re.p, P->d_im.p, s);
  GBTN_CUDA(cudaMemcpyAsync(re, P->d_re.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  GBTN_CUDA(cudaMemcpyAsync(im, P->d_im.p, sizeof(double), cudaMemcpyDeviceToHost, s));
  GBTN_CUDA(cudaStreamSynchronize(s));
  QN_CATCH(C)
}

}  // extern "C"
