// C-ABI layer of libgbtn: context and plan bookkeeping, argument validation,
// and the launch sequences behind update / environment / expect / logscalar /
// rescale.  No exception crosses the ABI: every entry point returns a status
// and records a message for gbtn_last_error.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <map>
#include <memory>
#include <mutex>
#include <numeric>
#include <type_traits>

#include "gbtn_internal.h"

namespace gbtn {
void upload_schedules(const DeviceSched& s);
}

using namespace gbtn;

struct gbtn_ctx {
  int device = 0;
  cudaStream_t own = nullptr;
  cudaStream_t stream = nullptr;
  std::string err;
  DeviceSched sched{};
  // optional per-kernel-class event timing (gbtn_ctx_set_profiling)
  int profiling = 0;
  struct Rec {
    int cls;
    cudaEvent_t a, b;
  };
  std::vector<Rec> recs;
};

namespace {

thread_local std::string g_err_noctx;

template <typename T>
struct DevBuf {
  T* p = nullptr;
  size_t n = 0;
  DevBuf() = default;
  DevBuf(const DevBuf&) = delete;
  DevBuf& operator=(const DevBuf&) = delete;
  ~DevBuf() {
    if (p) cudaFree(p);
  }
  void alloc(size_t count) {
    if (p) cudaFree(p);
    p = nullptr;
    n = count;
    if (count) GBTN_CUDA(cudaMalloc(&p, count * sizeof(T)));
  }
  void upload(const std::vector<T>& h, cudaStream_t s) {
    alloc(h.size());
    if (!h.empty()) GBTN_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  }
};

// Tensor-core work list: one record per vertex, in list order.
struct TcList {
  TcRec* d_recs = nullptr;
  int count = 0;
};

struct HostWork {
  std::vector<int> vertices;
  int ncap = 0, maxdeg = 0, team = 32;
};

}  // namespace

constexpr int kUploadChunks = 8;  // pieces of a host factor upload that overlap the image builds

struct gbtn_plan {
  gbtn_ctx* ctx = nullptr;
  int nv = 0, ne = 0, nnet = 1;
  bool sep_bra = false;
  bool cplx = false;  // complex tensors: arrays hold interleaved (re, im) doubles
  int es() const { return cplx ? 2 : 1; }  // doubles per element
  long long n_fac = 0, n_msg = 0, n_rdm = 0;
  int ncap = 0, maxdeg = 0;
  std::vector<VDesc> vd;
  std::vector<int> eu, ev, dchi, dsite, vnet;
  std::vector<long long> msg_off, rdm_off;
  std::vector<int> color;

  DevBuf<VDesc> d_vd;
  DevBuf<long long> d_msg_off, d_rdm_off;
  DevBuf<int> d_dchi, d_dsite;
  DevBuf<double> d_fac, d_bra;
  DevBuf<float> d_fac32, d_bra32;
  bool fac32_valid = false;
  DevBuf<double> d_msg[2];
  DevBuf<float> d_msg32[2];
  int cur = 0;  // buffer holding the current messages
  DevBuf<double> d_diffs, d_mean, d_rdm, d_edge_sc, d_re, d_im, d_scale, d_out;
  DevBuf<int> d_conv, d_iters, d_since, d_nconv;
  int* h_nconv = nullptr;  // pinned [2]: converged-network counts read while sweeping
  cudaEvent_t poll_ev[2] = {nullptr, nullptr};
  DevBuf<double> d_best;
  DevBuf<int> d_net_de_ptr, d_net_de, d_net_v_ptr, d_net_v, d_net_e_ptr, d_net_e;
  // work lists: index 0 = all vertices, 1.. = colour classes; two size classes each
  std::vector<std::pair<WorkList, WorkList>> lists;
  std::vector<std::unique_ptr<DevBuf<int>>> list_store;
  // tensor-core split of every list: vertices routed to the tensor-core
  // kernel (padded to degree 4, chi = 8; bra = ket) and the rest, which run
  // the FP32 SIMT kernel.  Candidates (tc_paddable) own an image slot; the
  // policy (and, for GBTN_TC_AUTO, the autotuner) chooses which of them use it.
  std::vector<TcList> tc_lists;
  std::vector<std::pair<WorkList, WorkList>> rest_lists;
  std::vector<std::unique_ptr<DevBuf<int>>> tc_store;
  std::vector<std::unique_ptr<DevBuf<TcRec>>> tc_rec_store;
  std::vector<int> tc_slot_vertex, tc_vslot;
  std::vector<TcRec> tc_recs;  // by slot
  std::vector<char> tc_cand, tc_use;
  int tc_policy = GBTN_TC_AUTO;
  bool tc_tuned = false;
  // SIMT team width per arithmetic and size class (0: the fixed rule), measured
  // before the first parallel or coloured sweeps of each arithmetic
  int simt_tuning = 1;
  bool team_tuned[5] = {};
  int team_pick[5][32] = {};
  int ncol = 0;
  double tc_tune_best_ms = 0.0;
  DevBuf<int> d_tc_slot_vertex, d_err;
  DevBuf<__nv_bfloat16> d_zimg;
  bool zimg_valid = false;
  // CUDA graphs of two sweeps (gbtn_plan_set_graphs), keyed by the launch
  // parameters; list_version changes whenever the work lists are rebuilt
  int graphs = 0;
  int list_version = 0;
  std::map<std::tuple<int, int, int, int, int, int, int, double>, std::pair<cudaGraph_t, cudaGraphExec_t>> graph_cache;
  void clear_graphs() {
    for (auto& kv : graph_cache) {
      if (kv.second.second) cudaGraphExecDestroy(kv.second.second);
      if (kv.second.first) cudaGraphDestroy(kv.second.first);
    }
    graph_cache.clear();
  }
  // overlapped factor upload: copy and image-build streams, one event per chunk
  cudaStream_t up_copy = nullptr, up_build = nullptr;
  cudaEvent_t up_ev[kUploadChunks + 1] = {};
  ~gbtn_plan() {
    clear_graphs();
    if (h_nconv) cudaFreeHost(h_nconv);
    for (cudaEvent_t e : poll_ev)
      if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : up_ev)
      if (e) cudaEventDestroy(e);
    if (up_copy) cudaStreamDestroy(up_copy);
    if (up_build) cudaStreamDestroy(up_build);
  }
  // global-memory path (bp_large.cu) for vertices beyond the shared-memory
  // kernels: per work list (0 = all, 1.. = colour classes), waves of vertices
  // of one degree whose scratch buffers fit kLargeWaveBytes together
  struct LargeWave {
    int k = 0, count = 0, max_tiles = 0, max_chi = 0;
    long long vstride = 0, scratch_elems = 0;
    std::vector<int> verts;
    DevBuf<int> d_verts;
    DevBuf<long long> d_off;
  };
  std::vector<char> is_large;
  bool has_large = false;
  std::vector<std::vector<std::unique_ptr<LargeWave>>> large_lists;
  long long large_scratch_elems = 0, large_partial_elems = 0;
  DevBuf<double> d_large_scratch, d_large_partial;  // sized in elements of the plan's widest arithmetic
  DevBuf<int> d_iota;                               // vertex ids 0..nv-1 (single-vertex waves)
  DevBuf<long long> d_zero_off;                     // scratch offset 0
  // sequential schedule in waves: the per-network sequences the waves were cut
  // for, and per wave the jobs of small (team 32) and larger (team 256) vertices
  std::vector<int> wave_key;  // per network: its length, then (vertex, leg) pairs
  std::vector<std::pair<WaveJobs, WaveJobs>> waves;
  DevBuf<int4> d_wave_jobs;
  DevBuf<int> d_wave_ptr, d_wave_iota;
  DevBuf<double> d_pos_diffs;
  int wave_version = 0;
  // host <-> device traffic of the plan's arrays (gbtn_plan_counters)
  long long cnt_fac_up = 0, cnt_msg_up = 0, cnt_msg_down = 0, cnt_fac_down = 0;
  // sweeps per phase of the last run (max over networks): BF16, FP32, refinement, FP64
  DevBuf<int> d_phase_iters;  // 4 x nnet
  int phase_fixed[4] = {0, 0, 0, 0};  // sweeps of a phase run without a tolerance (all of its maxiter)
  DevBuf<int> d_jobs;
  DevBuf<long long> d_half_off;
  DevBuf<double> d_halves;
};

namespace {

// The interleaved (re, im) doubles of a complex plan's arrays as elements.
inline zdouble* zptr(double* p) { return reinterpret_cast<zdouble*>(p); }
inline zfloat* zfptr(float* p) { return reinterpret_cast<zfloat*>(p); }
// An interleaved double buffer as elements of T (double, or zdouble for complex plans).
template <typename T>
inline T* as(double* p) { return reinterpret_cast<T*>(p); }
template <typename T>
inline const T* as(const double* p) { return reinterpret_cast<const T*>(p); }

// Arithmetic tag of the double-FP32 sweeps (FP64 storage, df32 arithmetic).
struct DF32 {};

// arithmetic -> (graph-cache tag, kernel class of the profiling API)
template <typename T> struct ElemTraits;
template <> struct ElemTraits<double> { static constexpr int tag = 0; static constexpr int kcls = GBTN_KCLASS_SIMT_F64; };
template <> struct ElemTraits<float> { static constexpr int tag = 1; static constexpr int kcls = GBTN_KCLASS_SIMT_F32; };
template <> struct ElemTraits<zdouble> { static constexpr int tag = 3; static constexpr int kcls = GBTN_KCLASS_SIMT_F64; };
template <> struct ElemTraits<zfloat> { static constexpr int tag = 4; static constexpr int kcls = GBTN_KCLASS_SIMT_F32; };
template <> struct ElemTraits<DF32> { static constexpr int tag = 5; static constexpr int kcls = GBTN_KCLASS_SIMT_DF32; };

// Large-path arithmetic code of (storage T, arithmetic A).
template <typename T, typename A> struct ArithOf;
template <> struct ArithOf<double, double> { static constexpr int value = kArithF64; };
template <> struct ArithOf<float, float> { static constexpr int value = kArithF32; };
template <> struct ArithOf<double, DF32> { static constexpr int value = kArithDF32; };
template <> struct ArithOf<zdouble, zdouble> { static constexpr int value = kArithZ64; };
template <> struct ArithOf<zfloat, zfloat> { static constexpr int value = kArithZ32; };

// One vertex-kernel launch in arithmetic A on storage T (A = T except for DF32).
template <typename T, typename A>
void launch_vertices(const WorkList& wl, const VDesc* vd, const T* fac, const T* bra, const T* in, T* out,
                     const long long* msg_off, double* diffs, const int* conv, int normalize, int want_diff,
                     cudaStream_t s) {
  if constexpr (std::is_same<A, DF32>::value)
    launch_bp_vertices_df32(wl, vd, fac, bra, in, out, msg_off, diffs, conv, normalize, want_diff, s);
  else
    launch_bp_vertices<T>(wl, vd, fac, bra, in, out, msg_off, diffs, conv, normalize, want_diff, s);
}

constexpr int kSmallN = 1024;  // vertices with n <= kSmallN run one per warp
// Reduced-precision phases stop at their noise floor: after this many sweeps
// without a new best mean diff below 0.9x the previous one.
constexpr int kStallSweeps = 3;

// Brackets one kernel launch with CUDA events when the context profiles.
struct KTimer {
  gbtn_ctx* c;
  int cls;
  cudaEvent_t a = nullptr;
  KTimer(gbtn_ctx* ctx, int k, bool active = true) : c(ctx), cls(k) {
    if (c->profiling && active) {
      GBTN_CUDA(cudaEventCreate(&a));
      GBTN_CUDA(cudaEventRecord(a, c->stream));
    }
  }
  ~KTimer() {
    if (!a) return;
    cudaEvent_t b = nullptr;
    if (cudaEventCreate(&b) == cudaSuccess && cudaEventRecord(b, c->stream) == cudaSuccess)
      c->recs.push_back({cls, a, b});
  }
};

void set_err(const gbtn_ctx* ctx, const std::string& m) {
  if (ctx)
    const_cast<gbtn_ctx*>(ctx)->err = m;
  else
    g_err_noctx = m;
}

#define API_TRY try {
#define API_CATCH(CTX)                                      \
  }                                                         \
  catch (const InvalidArg& e) {                             \
    set_err(CTX, e.what());                                 \
    return GBTN_ERR_INVALID;                                \
  }                                                         \
  catch (const Unsupported& e) {                            \
    set_err(CTX, e.what());                                 \
    return GBTN_ERR_UNSUPPORTED;                            \
  }                                                         \
  catch (const Timeout& e) {                                \
    set_err(CTX, e.what());                                 \
    return GBTN_ERR_TIMEOUT;                                \
  }                                                         \
  catch (const CudaError& e) {                              \
    set_err(CTX, e.what());                                 \
    return GBTN_ERR_CUDA;                                   \
  }                                                         \
  catch (const std::bad_alloc&) {                           \
    set_err(CTX, "host allocation failed");                 \
    return GBTN_ERR_NOMEM;                                  \
  }                                                         \
  catch (const std::exception& e) {                         \
    set_err(CTX, e.what());                                 \
    return GBTN_ERR_INVALID;                                \
  }                                                         \
  return GBTN_OK;

void require(bool c, const std::string& m) {
  if (!c) throw InvalidArg(m);
}

WorkList make_list(gbtn_plan* P, const std::vector<int>& verts_in, int team,
                   std::vector<std::unique_ptr<DevBuf<int>>>* store = nullptr) {
  // size classes: team 32 up to 128, 256, 512, 1024 elements; team 256 up to
  // 2048, 4096, 8192, 16384, ... (one launch each, shared memory per class)
  std::vector<int> verts = verts_in;
  std::stable_sort(verts.begin(), verts.end(), [&](int a, int b) { return P->vd[a].n < P->vd[b].n; });
  WorkList w;
  w.count = (int)verts.size();
  w.team = team;
  long long bound = team == 32 ? 128 : 2048;
  for (int i = 0; i < w.count;) {
    while (P->vd[verts[i]].n > bound) bound *= 2;
    const bool last = w.nsub == kMaxSub - 1;  // the last class takes every remaining vertex
    int j = i;
    int ncap = 0, maxdeg = 0;
    while (j < w.count && (last || P->vd[verts[j]].n <= bound)) {
      ncap = std::max(ncap, P->vd[verts[j]].n);
      maxdeg = std::max(maxdeg, P->vd[verts[j]].k);
      ++j;
    }
    w.sub_begin[w.nsub] = i;
    w.sub_count[w.nsub] = j - i;
    w.sub_ncap[w.nsub] = ncap;
    w.sub_maxdeg[w.nsub] = maxdeg;
    w.nsub++;
    i = j;
    bound *= 2;
  }
  for (int v : verts) {
    w.ncap = std::max(w.ncap, P->vd[v].n);
    w.maxdeg = std::max(w.maxdeg, P->vd[v].k);
  }
  auto buf = std::make_unique<DevBuf<int>>();
  buf->upload(verts, P->ctx->stream);
  w.d_vertices = buf->p;
  (store ? *store : P->list_store).push_back(std::move(buf));
  return w;
}

std::pair<WorkList, WorkList> split_list(gbtn_plan* P, const std::vector<int>& verts,
                                         std::vector<std::unique_ptr<DevBuf<int>>>* store = nullptr) {
  std::vector<int> small, large;
  for (int v : verts) {
    if (!P->is_large.empty() && P->is_large[v]) continue;  // the global-memory path takes these
    (P->vd[v].n <= kSmallN ? small : large).push_back(v);
  }
  return {make_list(P, small, 32, store), make_list(P, large, 256, store)};
}

void copy_out(gbtn_plan* P, void* dst, const void* src, size_t bytes, int mem) {
  GBTN_CUDA(cudaMemcpyAsync(dst, src, bytes, mem == GBTN_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                            P->ctx->stream));
  if (mem == GBTN_HOST) GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));
}

void copy_in(gbtn_plan* P, void* dst, const void* src, size_t bytes, int mem) {
  GBTN_CUDA(cudaMemcpyAsync(dst, src, bytes, mem == GBTN_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                            P->ctx->stream));
  if (mem == GBTN_HOST) GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));
}

// FP32 message buffers (and room for FP32 factors).
void ensure_f32_bufs(gbtn_plan* P) {
  if (!P->d_fac32.p) {  // floats per element: 1, or 2 for complex networks (zfloat)
    P->d_fac32.alloc(P->es() * P->n_fac);
    if (P->sep_bra) P->d_bra32.alloc(P->es() * P->n_fac);
    P->d_msg32[0].alloc(P->es() * P->n_msg);
    P->d_msg32[1].alloc(P->es() * P->n_msg);
  }
}

// FP32 buffers and the FP32 copy of the factors (the FP32 SIMT kernel's input).
void ensure_f32(gbtn_plan* P) {
  cudaStream_t s = P->ctx->stream;
  ensure_f32_bufs(P);
  if (!P->fac32_valid) {
    launch_convert_f64_to_f32(P->d_fac.p, P->d_fac32.p, P->es() * P->n_fac, s);
    if (P->sep_bra) launch_convert_f64_to_f32(P->d_bra.p, P->d_bra32.p, P->es() * P->n_fac, s);
    P->fac32_valid = true;
  }
}

// Shared memory of one team of the SIMT kernels for a tensor of n elements
// (padded layout: one unused element per 32, see spos in bp_device.cuh).
size_t smem_need(int n, int k, bool sep_bra, size_t elt, int team) {
  const int nbuf = k <= 4 ? 3 : kNumBufs;
  const size_t np = (size_t)n + (n >> 5) + 1;
  size_t b = (sizeof(VDesc) + 15) / 16 * 16;
  b += elt * (np * (nbuf + (sep_bra ? 1 : 0)) + team_tail_elems(team));
  return (b + 15) / 16 * 16;
}

using GraphKey = std::tuple<int, int, int, int, int, int, int, double>;

// Convergence polling while sweeping.  Each poll queues a 4-byte copy of the
// converged-network count (kept on the device by reduce_diffs) into pinned
// memory and records an event, then waits for the PREVIOUS poll's event and
// reads its count -- so the GPU always has the sweeps since the last poll
// queued while the host waits, and the loop overshoots convergence by at most
// two poll periods.
struct ConvPoll {
  gbtn_plan* P;
  int n = 0;
  explicit ConvPoll(gbtn_plan* p) : P(p) {}
  bool done() {
    const int slot = n & 1;
    GBTN_CUDA(cudaMemcpyAsync(P->h_nconv + slot, P->d_nconv.p, sizeof(int), cudaMemcpyDeviceToHost, P->ctx->stream));
    GBTN_CUDA(cudaEventRecord(P->poll_ev[slot], P->ctx->stream));
    if (++n < 2) return false;
    GBTN_CUDA(cudaEventSynchronize(P->poll_ev[slot ^ 1]));
    return P->h_nconv[slot ^ 1] >= P->nnet;
  }
};

// maxiter sweeps of `sweep`.  With graphs on (and no per-launch profiling),
// the first sweep runs as plain launches and the rest are replays of one CUDA
// graph holding two sweeps -- after two sweeps the double-buffer parity is
// back where it started, so the same graph serves every pair.  The graph is
// kept in the plan under `key` (launch parameters, buffer parity, list
// version) and reused by later calls.  With `poll`, the converged-network
// count is polled every two sweeps and the loop ends once every network has
// converged (the remaining sweeps would only carry the messages forward).
template <class F>
void sweep_loop(gbtn_plan* P, int maxiter, const GraphKey& key, F&& sweep, bool poll = false) {
  cudaStream_t s = P->ctx->stream;
  int it = 0;
  ConvPoll cp(P);
  if (P->graphs && !P->ctx->profiling && maxiter >= 3) {
    sweep();
    ++it;
    auto found = P->graph_cache.find(key);
    if (found == P->graph_cache.end()) {
      cudaGraph_t g = nullptr;
      cudaGraphExec_t ge = nullptr;
      GBTN_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      try {
        sweep();
        sweep();
      } catch (...) {
        cudaStreamEndCapture(s, &g);
        if (g) cudaGraphDestroy(g);
        throw;
      }
      GBTN_CUDA(cudaStreamEndCapture(s, &g));
      const cudaError_t e = cudaGraphInstantiate(&ge, g, 0);
      if (e != cudaSuccess) {
        cudaGraphDestroy(g);
        GBTN_CUDA(e);
      }
      found = P->graph_cache.emplace(key, std::make_pair(g, ge)).first;
    }
    for (; it + 2 <= maxiter; it += 2) {
      GBTN_CUDA(cudaGraphLaunch(found->second.second, s));
      if (poll && it + 2 < maxiter && cp.done()) return;
    }
  }
  for (; it < maxiter; ++it) {
    sweep();
    if (poll && (it & 1) && it + 1 < maxiter && cp.done()) return;
  }
}

void run_large(gbtn_plan* P, size_t li, int arith, const void* fac, const void* bra, const void* in, void* out,
               const int* conv, int normalize, int want_diff, cudaStream_t s);

// A work list carrying the measured team widths of arithmetic `arith`.
WorkList picked(const WorkList& w, const gbtn_plan* P, int arith) {
  WorkList c = w;
  c.pick = P->team_pick[arith];
  return c;
}

// The measured autotuner of the SIMT sweeps, keyed on the vertex shapes: for
// every size class of the parallel work lists (vertex size n up to a power of
// two, which with the degree fixes chi^k d), time one launch of each team
// width that fits shared memory -- 32 (four vertices per block), 128 or 256
// threads per vertex -- on up to 2048 of the class's own vertices with CUDA
// events (best of two after a warm-up), and keep the fastest for that class.
// The launches read `in` and write `out` (a message buffer the next sweep
// overwrites), with no convergence flags.
template <typename T, typename A>
void tune_teams(gbtn_plan* P, const T* fac, const T* bra, const T* in, T* out) {
  constexpr int arith = ArithOf<T, A>::value;
  if (P->team_tuned[arith]) return;
  P->team_tuned[arith] = true;
  if (!P->simt_tuning) return;
  cudaStream_t s = P->ctx->stream;
  const size_t elt = std::is_same<A, DF32>::value ? 8 : sizeof(T);
  cudaEvent_t e0, e1;
  GBTN_CUDA(cudaEventCreate(&e0));
  GBTN_CUDA(cudaEventCreate(&e1));
  bool changed = false;
  for (const WorkList* lst : {&P->lists[0].first, &P->lists[0].second}) {
    for (int c = 0; c < lst->nsubs(); ++c) {
      WorkList w = lst->sub(c);
      if (w.count == 0) continue;
      const int key = WorkList::class_key(w.ncap);
      if (P->team_pick[arith][key] != 0) continue;  // tuned on another list's class of this size
      w.count = std::min(w.count, 2048);
      float best = 0.f;
      int best_team = 0;
      for (int team : {32, 128, 256}) {
        const size_t sm = smem_need(w.ncap, w.maxdeg, bra != nullptr, elt, team) * (team == 32 ? 4 : 1);
        if (sm > 227 * 1024) continue;
        if (P->simt_tuning != 1) {  // one width forced wherever it fits
          if (team == P->simt_tuning) best_team = team;
          continue;
        }
        w.team = team;
        float t = 0.f;
        for (int rep = 0; rep < 3; ++rep) {
          GBTN_CUDA(cudaEventRecord(e0, s));
          launch_vertices<T, A>(w, P->d_vd.p, fac, bra, in, out, P->d_msg_off.p, P->d_diffs.p, nullptr, 1, 1, s);
          GBTN_CUDA(cudaEventRecord(e1, s));
          GBTN_CUDA(cudaEventSynchronize(e1));
          float ms = 0.f;
          GBTN_CUDA(cudaEventElapsedTime(&ms, e0, e1));
          if (rep == 1 || (rep == 2 && ms < t)) t = ms;
        }
        if (best_team == 0 || t < best) {
          best = t;
          best_team = team;
        }
      }
      if (best_team != 0) {
        P->team_pick[arith][key] = best_team;
        changed = true;
      }
    }
  }
  GBTN_CUDA(cudaEventDestroy(e0));
  GBTN_CUDA(cudaEventDestroy(e1));
  if (changed) ++P->list_version;  // graphs captured before the choice are stale
}

// Sweeps of the parallel or coloured schedule on storage T in arithmetic A.
template <typename T, typename A = T>
void run_sweeps(gbtn_plan* P, int schedule, int maxiter, double tol, int normalize, T* msg0, T* msg1, const T* fac,
                const T* bra, int& cur, int stall = 0) {
  cudaStream_t s = P->ctx->stream;
  const bool want_diff = tol >= 0.0;
  GBTN_CUDA(cudaMemsetAsync(P->d_conv.p, 0, sizeof(int) * P->nnet, s));
  GBTN_CUDA(cudaMemsetAsync(P->d_iters.p, 0, sizeof(int) * P->nnet, s));
  GBTN_CUDA(cudaMemsetAsync(P->d_nconv.p, 0, sizeof(int), s));
  const int* conv = want_diff ? P->d_conv.p : nullptr;
  T* msg[2] = {msg0, msg1};
  constexpr int arith = ArithOf<T, A>::value;
  tune_teams<T, A>(P, fac, bra, msg[cur], msg[cur ^ 1]);
  const GraphKey key{ElemTraits<A>::tag, schedule, normalize, want_diff ? 1 : 0, stall, cur, P->list_version, tol};
  constexpr int kcls = ElemTraits<A>::kcls;
  sweep_loop(P, maxiter, key, [&] {
    if (schedule == GBTN_SCHED_PARALLEL) {
      const T* in = msg[cur];
      T* out = msg[cur ^ 1];
      {
        KTimer kt(P->ctx, kcls, P->lists[0].first.count > 0);
        launch_vertices<T, A>(picked(P->lists[0].first, P, arith), P->d_vd.p, fac, bra, in, out, P->d_msg_off.p,
                              P->d_diffs.p, conv, normalize, want_diff, s);
      }
      {
        KTimer kt(P->ctx, kcls, P->lists[0].second.count > 0);
        launch_vertices<T, A>(picked(P->lists[0].second, P, arith), P->d_vd.p, fac, bra, in, out, P->d_msg_off.p,
                              P->d_diffs.p, conv, normalize, want_diff, s);
      }
      {
        KTimer kt(P->ctx, GBTN_KCLASS_LARGE, P->has_large);
        run_large(P, 0, ArithOf<T, A>::value, fac, bra, in, out, conv, normalize, want_diff, s);
      }
      cur ^= 1;
    } else {
      for (size_t c = 1; c < P->lists.size(); ++c) {
        T* m = msg[cur];
        launch_vertices<T, A>(picked(P->lists[c].first, P, arith), P->d_vd.p, fac, bra, m, m, P->d_msg_off.p,
                              P->d_diffs.p, conv, normalize, want_diff, s);
        launch_vertices<T, A>(picked(P->lists[c].second, P, arith), P->d_vd.p, fac, bra, m, m, P->d_msg_off.p,
                              P->d_diffs.p, conv, normalize, want_diff, s);
        run_large(P, c, ArithOf<T, A>::value, fac, bra, m, m, conv, normalize, want_diff, s);
      }
    }
    if (want_diff)
      launch_reduce_diffs(P->nnet, P->d_net_de_ptr.p, P->d_net_de.p, P->d_diffs.p, tol, P->d_conv.p, P->d_iters.p,
                          P->d_mean.p, s, stall, P->d_best.p, P->d_since.p, P->d_nconv.p);
  }, want_diff);
}

// Raise the device-side error word (set by a bounded wait that gave up).
void check_device_error(gbtn_plan* P) {
  int e = 0;
  GBTN_CUDA(cudaMemcpyAsync(&e, P->d_err.p, sizeof(int), cudaMemcpyDeviceToHost, P->ctx->stream));
  GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));
  if (e != 0) {
    GBTN_CUDA(cudaMemsetAsync(P->d_err.p, 0, sizeof(int), P->ctx->stream));
    throw Timeout("tensor-core sweep: a bounded device wait gave up (TMA copy or MMA did not complete)");
  }
}

void ensure_zimg(gbtn_plan* P) {
  const int n = (int)P->tc_slot_vertex.size();
  if (n == 0) return;
  if (!P->d_zimg.p) P->d_zimg.alloc((size_t)n * 8192);
  if (!P->zimg_valid) {
    launch_build_zimg(P->d_tc_slot_vertex.p, n, P->d_vd.p, P->d_fac.p, P->d_zimg.p, P->ctx->stream);
    P->zimg_valid = true;
  }
}

// Algorithmic flops of all outgoing messages of a vertex: k messages of
// 2 d prod(chi) sum(chi) each (updated_message, abstractbeliefpropagationcache.jl:225-239).
double vertex_flops(const VDesc& d) {
  double sc = 0.0;
  for (int p = 0; p < d.k; ++p) sc += d.chi[p];
  return d.k * 2.0 * d.n * sc;
}

// Image slots and records for every candidate vertex.
void build_tc_slots(gbtn_plan* P) {
  cudaStream_t s = P->ctx->stream;
  P->tc_vslot.assign(P->nv, -1);
  P->tc_slot_vertex.clear();
  P->tc_recs.clear();
  for (int v = 0; v < P->nv; ++v)
    if (P->tc_cand[v]) {
      P->tc_vslot[v] = (int)P->tc_slot_vertex.size();
      P->tc_slot_vertex.push_back(v);
      TcRec r = tc_record(P->vd[v], P->msg_off);
      r.slot = P->tc_vslot[v];
      P->tc_recs.push_back(r);
    }
  std::vector<int> sv = P->tc_slot_vertex;
  if (sv.empty()) sv.push_back(0);
  P->d_tc_slot_vertex.upload(sv, s);
  P->zimg_valid = false;
}

TcList make_tc_list(gbtn_plan* P, const std::vector<int>& verts, std::vector<std::unique_ptr<DevBuf<TcRec>>>& store) {
  std::vector<TcRec> recs;
  recs.reserve(verts.size());
  for (int v : verts) recs.push_back(P->tc_recs[P->tc_vslot[v]]);
  auto buf = std::make_unique<DevBuf<TcRec>>();
  buf->upload(recs, P->ctx->stream);
  TcList l;
  l.d_recs = buf->p;
  l.count = (int)verts.size();
  store.push_back(std::move(buf));
  return l;
}

// Work lists (all vertices, then every colour class) for the split `use`.
void build_tc_lists(gbtn_plan* P, const std::vector<char>& use) {
  GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));  // no launch still reads the old lists
  P->clear_graphs();
  ++P->list_version;
  P->tc_use = use;
  P->tc_lists.clear();
  P->rest_lists.clear();
  P->tc_store.clear();
  P->tc_rec_store.clear();
  for (int li = 0; li <= P->ncol; ++li) {
    std::vector<int> tcv, rest;
    for (int v = 0; v < P->nv; ++v) {
      if (li > 0 && P->color[v] != li - 1) continue;
      (use[v] ? tcv : rest).push_back(v);
    }
    P->tc_lists.push_back(make_tc_list(P, tcv, P->tc_rec_store));
    P->rest_lists.push_back(split_list(P, rest, &P->tc_store));
  }
}

template <class F>
float time_ms(cudaStream_t s, F&& fn, int reps) {
  cudaEvent_t a = nullptr, b = nullptr;
  GBTN_CUDA(cudaEventCreate(&a));
  GBTN_CUDA(cudaEventCreate(&b));
  fn();  // warm-up
  GBTN_CUDA(cudaEventRecord(a, s));
  for (int r = 0; r < reps; ++r) fn();
  GBTN_CUDA(cudaEventRecord(b, s));
  GBTN_CUDA(cudaEventSynchronize(b));
  float ms = 0.f;
  GBTN_CUDA(cudaEventElapsedTime(&ms, a, b));
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  return ms / reps;
}

// Choose which candidates run on the tensor cores.  GBTN_TC_AUTO measures:
// candidates sorted by algorithmic flops are split at a point q (the q
// smallest on the FP32 SIMT kernel, the rest on the tensor-core kernel --
// padding makes the tensor-core cost per vertex independent of its shape,
// while the SIMT cost grows with it), both launches of every split are timed
// on this plan's own vertices and messages, and the fastest split is kept
// (split points 0, 1/4, .., 1, then +-1/8 around the best).  The FP32
// messages of the current state must be in msg32[0].
void tune_tc_split(gbtn_plan* P) {
  if (P->tc_tuned) return;
  const int nv = P->nv;
  std::vector<char> use(nv, 0);
  if (P->tc_policy == GBTN_TC_ALL) {
    use = P->tc_cand;
  } else if (P->tc_policy == GBTN_TC_NATIVE) {
    for (int v = 0; v < nv; ++v) use[v] = P->tc_cand[v] && tc_native(P->vd[v]);
  } else if (P->tc_policy == GBTN_TC_AUTO) {
    ensure_f32(P);  // the timed SIMT launches read the FP32 factors
    std::vector<int> cv;
    for (int v = 0; v < nv; ++v)
      if (P->tc_cand[v]) cv.push_back(v);
    if (!cv.empty()) {
      std::stable_sort(cv.begin(), cv.end(),
                       [&](int a, int b) { return vertex_flops(P->vd[a]) < vertex_flops(P->vd[b]); });
      cudaStream_t s = P->ctx->stream;
      ensure_zimg(P);
      DevBuf<float> out;
      out.alloc(P->n_msg);
      const float* in = P->d_msg32[0].p;
      const int N = (int)cv.size();
      std::map<int, double> cost;  // split index -> measured ms
      auto measure = [&](int k) {
        if (cost.count(k)) return;
        std::vector<std::unique_ptr<DevBuf<int>>> store;
        std::vector<std::unique_ptr<DevBuf<TcRec>>> rstore;
        const std::vector<int> lo(cv.begin(), cv.begin() + k), hi(cv.begin() + k, cv.end());
        const std::pair<WorkList, WorkList> sl = split_list(P, lo, &store);
        const TcList th = make_tc_list(P, hi, rstore);
        double ms = 0.0;
        if (!lo.empty())
          ms += time_ms(s, [&] {
            launch_bp_vertices<float>(sl.first, P->d_vd.p, P->d_fac32.p, nullptr, in, out.p, P->d_msg_off.p,
                                      P->d_diffs.p, nullptr, 1, 1, s);
            launch_bp_vertices<float>(sl.second, P->d_vd.p, P->d_fac32.p, nullptr, in, out.p, P->d_msg_off.p,
                                      P->d_diffs.p, nullptr, 1, 1, s);
          }, 3);
        if (!hi.empty())
          ms += time_ms(s, [&] {
            launch_tc_vertices(th.d_recs, th.count, P->d_zimg.p, in, out.p,
                               P->d_diffs.p, nullptr, 1, 1, P->d_err.p, s);
          }, 3);
        cost[k] = ms;
      };
      int best = 0;
      for (int q = 0; q <= 4; ++q) measure((int)((long long)N * q / 4));
      for (auto& kv : cost)
        if (kv.second < cost[best]) best = kv.first;
      for (int d : {-1, 1}) measure(std::min(N, std::max(0, best + d * N / 8)));
      for (auto& kv : cost)
        if (kv.second < cost[best]) best = kv.first;
      P->tc_tune_best_ms = cost[best];
      for (int i = best; i < N; ++i) use[cv[i]] = 1;
      check_device_error(P);
    }
  }
  build_tc_lists(P, use);
  P->tc_tuned = true;
}

// Does the BF16 sweep run any vertex on the FP32 SIMT kernel?
bool bf16_has_simt(const gbtn_plan* P) {
  if (P->has_large) return true;  // large vertices run the FP32 global-memory path
  for (const auto& l : P->rest_lists)
    if (l.first.count > 0 || l.second.count > 0) return true;
  return false;
}

// BF16 sweeps (parallel or coloured): tensor-core kernel on the eligible
// vertices, FP32 SIMT kernel on the rest, FP32 messages.
void run_sweeps_bf16(gbtn_plan* P, int schedule, int maxiter, double tol, int normalize, int& c32, int stall = 0) {
  cudaStream_t s = P->ctx->stream;
  const bool want_diff = tol >= 0.0;
  GBTN_CUDA(cudaMemsetAsync(P->d_conv.p, 0, sizeof(int) * P->nnet, s));
  GBTN_CUDA(cudaMemsetAsync(P->d_iters.p, 0, sizeof(int) * P->nnet, s));
  GBTN_CUDA(cudaMemsetAsync(P->d_nconv.p, 0, sizeof(int), s));
  const int* conv = want_diff ? P->d_conv.p : nullptr;
  const float* fac = P->d_fac32.p;
  auto one = [&](size_t li, const float* in, float* out) {
    const TcList& tl = P->tc_lists[li];
    {
      KTimer kt(P->ctx, GBTN_KCLASS_TENSOR_CORE, tl.count > 0);
      launch_tc_vertices(tl.d_recs, tl.count, P->d_zimg.p, in, out, P->d_diffs.p,
                         conv, normalize, want_diff, P->d_err.p, s);
    }
    {
      KTimer kt(P->ctx, GBTN_KCLASS_SIMT_F32, P->rest_lists[li].first.count > 0);
      launch_bp_vertices<float>(P->rest_lists[li].first, P->d_vd.p, fac, nullptr, in, out, P->d_msg_off.p,
                                P->d_diffs.p, conv, normalize, want_diff, s);
    }
    {
      KTimer kt(P->ctx, GBTN_KCLASS_SIMT_F32, P->rest_lists[li].second.count > 0);
      launch_bp_vertices<float>(P->rest_lists[li].second, P->d_vd.p, fac, nullptr, in, out, P->d_msg_off.p,
                                P->d_diffs.p, conv, normalize, want_diff, s);
    }
    run_large(P, li, kArithF32, fac, nullptr, in, out, conv, normalize, want_diff, s);
  };
  const GraphKey key{2, schedule, normalize, want_diff ? 1 : 0, stall, c32, P->list_version, tol};
  sweep_loop(P, maxiter, key, [&] {
    if (schedule == GBTN_SCHED_PARALLEL) {
      one(0, P->d_msg32[c32].p, P->d_msg32[c32 ^ 1].p);
      c32 ^= 1;
    } else {
      for (size_t c = 1; c < P->tc_lists.size(); ++c) one(c, P->d_msg32[c32].p, P->d_msg32[c32].p);
    }
    if (want_diff)
      launch_reduce_diffs(P->nnet, P->d_net_de_ptr.p, P->d_net_de.p, P->d_diffs.p, tol, P->d_conv.p, P->d_iters.p,
                          P->d_mean.p, s, stall, P->d_best.p, P->d_since.p, P->d_nconv.p);
  }, want_diff);
}

void finish_iters(gbtn_plan* P, bool want_diff, int maxiter, int32_t* iters, double* mean_diff) {
  cudaStream_t s = P->ctx->stream;
  if (!iters && !mean_diff) return;
  check_device_error(P);
  std::vector<int> it(P->nnet, maxiter);
  std::vector<double> md(P->nnet, NAN);
  if (want_diff) {
    GBTN_CUDA(cudaMemcpyAsync(it.data(), P->d_iters.p, sizeof(int) * P->nnet, cudaMemcpyDeviceToHost, s));
    GBTN_CUDA(cudaMemcpyAsync(md.data(), P->d_mean.p, sizeof(double) * P->nnet, cudaMemcpyDeviceToHost, s));
  }
  GBTN_CUDA(cudaStreamSynchronize(s));
  if (iters) std::copy(it.begin(), it.end(), iters);
  if (mean_diff) std::copy(md.begin(), md.end(), mean_diff);
}

// Keep the per-network sweep counts of the phase that just ran (slot 0-3).
void record_phase(gbtn_plan* P, int slot) {
  GBTN_CUDA(cudaMemcpyAsync(P->d_phase_iters.p + (size_t)slot * P->nnet, P->d_iters.p, sizeof(int) * P->nnet,
                            cudaMemcpyDeviceToDevice, P->ctx->stream));
}

constexpr long long kLargeWaveBytes = 1LL << 30;  // scratch of one wave of large vertices

// Tiles and partial-sum elements of the fibers of one leg (p < 0: the site index).
void large_leg_cost(const VDesc& d, int p, int& tiles, long long& partial) {
  const int chi = p >= 0 ? d.chi[p] : d.d, st = p >= 0 ? d.st[p] : 1;
  const LegTiling g = leg_tiling(d.n, st, chi);
  tiles = g.ntl * g.ntj;
  partial = (long long)tiles * chi * chi;
}

// Scratch buffers of a large vertex: the schedule's, and at least two for the
// absorb chains of environments, updated_message and the sequential schedule.
int large_nbuf(const gbtn_ctx* C, int k) { return std::max(C->sched.nbuf[k], 3) - 1; }

// Waves of the large vertices among `verts`, grouped by degree.
std::vector<std::unique_ptr<gbtn_plan::LargeWave>> build_large_waves(gbtn_plan* P, const std::vector<int>& verts) {
  std::vector<std::unique_ptr<gbtn_plan::LargeWave>> out;
  const long long elt = P->cplx ? 16 : 8;
  for (int k = 0; k <= kMaxDeg; ++k) {
    std::unique_ptr<gbtn_plan::LargeWave> w;
    long long bytes = 0;
    auto flush = [&] {
      if (!w || w->count == 0) return;
      std::vector<long long> off;
      long long o = 0;
      for (int v : w->verts) {
        off.push_back(o);
        o += (long long)large_nbuf(P->ctx, k) * P->vd[v].n;
      }
      w->scratch_elems = o;
      w->d_verts.upload(w->verts, P->ctx->stream);
      w->d_off.upload(off, P->ctx->stream);
      P->large_scratch_elems = std::max(P->large_scratch_elems, o);
      P->large_partial_elems = std::max(P->large_partial_elems, w->vstride * w->count);
      out.push_back(std::move(w));
    };
    for (int v : verts) {
      if (!P->is_large[v] || P->vd[v].k != k) continue;
      const VDesc& d = P->vd[v];
      int mt = 0, mc = 0;
      long long vs = 0;
      for (int p = -1; p < d.k; ++p) {
        int t;
        long long pe;
        large_leg_cost(d, p, t, pe);
        mt = std::max(mt, t);
        vs = std::max(vs, pe);
        if (p >= 0) mc = std::max(mc, d.chi[p]);
      }
      const long long need = ((long long)large_nbuf(P->ctx, k) * d.n + vs) * elt;
      if (w && (bytes + need > kLargeWaveBytes || w->count >= 65535)) {
        flush();
        w.reset();
        bytes = 0;
      }
      if (!w) {
        w = std::make_unique<gbtn_plan::LargeWave>();
        w->k = k;
      }
      w->verts.push_back(v);
      w->count++;
      w->max_tiles = std::max(w->max_tiles, mt);
      w->max_chi = std::max(w->max_chi, mc);
      w->vstride = std::max(w->vstride, vs);
      bytes += need;
    }
    flush();
  }
  return out;
}

// Scratch and partial sums of one vertex processed alone (updated_message and
// the sequential schedule of plans with large vertices take any vertex).
void reserve_single_vertex(gbtn_plan* P) {
  for (int v = 0; v < P->nv; ++v) {
    const VDesc& d = P->vd[v];
    long long vs = 0;
    for (int p = -1; p < d.k; ++p) {
      int t;
      long long pe;
      large_leg_cost(d, p, t, pe);
      vs = std::max(vs, pe);
    }
    P->large_scratch_elems = std::max(P->large_scratch_elems, (long long)large_nbuf(P->ctx, d.k) * d.n);
    P->large_partial_elems = std::max(P->large_partial_elems, vs);
  }
}

void ensure_large_bufs(gbtn_plan* P) {
  const size_t dbl = P->cplx ? 2 : 1;  // doubles per element of the widest arithmetic
  if (!P->d_large_scratch.p && P->large_scratch_elems > 0) P->d_large_scratch.alloc(dbl * P->large_scratch_elems);
  if (!P->d_large_partial.p && P->large_partial_elems > 0) P->d_large_partial.alloc(dbl * P->large_partial_elems);
}

LargeArgs<double> large_args(const gbtn_plan::LargeWave& w, const gbtn_plan* P, const void* fac, const void* bra,
                             const void* msgs) {
  LargeArgs<double> a;
  a.verts = w.d_verts.p;
  a.buf_off = w.d_off.p;
  a.vd = P->d_vd.p;
  a.fac = static_cast<const double*>(fac);
  a.bra = static_cast<const double*>(bra);
  a.msgs = static_cast<const double*>(msgs);
  a.msg_off = P->d_msg_off.p;
  return a;
}

// Every outgoing message of the large vertices of work list li, in arithmetic
// `arith` (storage: double, float, zdouble or zfloat arrays).
void run_large(gbtn_plan* P, size_t li, int arith, const void* fac, const void* bra, const void* in, void* out,
               const int* conv, int normalize, int want_diff, cudaStream_t s) {
  if (!P->has_large || li >= P->large_lists.size()) return;
  ensure_large_bufs(P);
  for (const auto& w : P->large_lists[li]) {
    const LargeArgs<double> a = large_args(*w, P, fac, bra, in);
    const int len = P->ctx->sched.len[w->k];
    for (int i = 0; i < len; ++i)
      launch_large_op_any(arith, a, w->count, w->max_tiles, w->max_chi, P->ctx->sched.ops[w->k][i],
                          P->d_large_scratch.p, P->d_large_partial.p, w->vstride, in, out, P->d_diffs.p, conv,
                          normalize, want_diff, s);
  }
}

// The absorb chain of every leg but `skip` (ping-pong between scratch buffers
// 1 and 2, from the site tensor); returns the buffer holding the result.
int large_chain(const VDesc& d, int skip, std::vector<SchedOp>& ops) {
  int cur = 0;
  for (int p = 0; p < d.k; ++p) {
    if (p == skip) continue;
    const int nxt = cur == 1 ? 2 : 1;
    ops.push_back({0, (int8_t)cur, (int8_t)nxt, (int8_t)p});
    cur = nxt;
  }
  return cur;
}

// One-site RDMs of the large vertices (FP64 or complex FP64).
void large_rdms(gbtn_plan* P, const double* fac, const double* bra, const double* msgs, double* rdm) {
  if (!P->has_large) return;
  ensure_large_bufs(P);
  cudaStream_t s = P->ctx->stream;
  const int arith = P->cplx ? kArithZ64 : kArithF64;
  for (const auto& w : P->large_lists[0]) {
    const LargeArgs<double> a = large_args(*w, P, fac, bra, msgs);
    std::vector<SchedOp> ops;
    const int src = large_chain(P->vd[w->verts[0]], -1, ops);
    for (const SchedOp& op : ops)
      launch_large_op_any(arith, a, w->count, w->max_tiles, w->max_chi, op, P->d_large_scratch.p,
                          P->d_large_partial.p, w->vstride, msgs, nullptr, nullptr, nullptr, 0, 0, s);
    launch_large_rdm_any(arith, a, w->count, w->max_tiles, src, P->d_large_scratch.p, P->d_large_partial.p,
                         w->vstride, rdm, P->d_rdm_off.p, s);
  }
}

// One message of a vertex through the global-memory path: the absorb chain of
// every other leg, CLOSE on `leg`, normalised into out + msg_off[out_de]
// (message_diff into diffs when want_diff).  Used for single messages of large
// vertices and by the sequential schedule of plans that hold large vertices.
void large_one_message(gbtn_plan* P, int arith, int v, int leg, const void* fac, const void* bra, const void* msgs,
                       void* out, int normalize, int want_diff, cudaStream_t s) {
  ensure_large_bufs(P);
  const VDesc& d = P->vd[v];
  gbtn_plan::LargeWave w;
  w.count = 1;
  for (int p = -1; p < d.k; ++p) {
    int t;
    long long pe;
    large_leg_cost(d, p, t, pe);
    w.max_tiles = std::max(w.max_tiles, t);
    w.vstride = std::max(w.vstride, pe);
    if (p >= 0) w.max_chi = std::max(w.max_chi, d.chi[p]);
  }
  LargeArgs<double> a = large_args(w, P, fac, bra, msgs);
  a.verts = P->d_iota.p + v;
  a.buf_off = P->d_zero_off.p;
  std::vector<SchedOp> ops;
  const int src = large_chain(d, leg, ops);
  ops.push_back({1, (int8_t)src, 0, (int8_t)leg});
  for (const SchedOp& op : ops)
    launch_large_op_any(arith, a, 1, w.max_tiles, w.max_chi, op, P->d_large_scratch.p, P->d_large_partial.p,
                        w.vstride, msgs, out, P->d_diffs.p, nullptr, normalize, want_diff, s);
}

// Cut the per-network sequences into waves.  A job (one message) goes to the
// first wave after every job it depends on in sequence order: the last writer
// of each message it reads (read after write), the readers since the last
// write of the message it writes (write after read) and that last writer
// (write after write).  Networks are independent, so wave l holds level l of
// every network.
void build_waves(gbtn_plan* P, const std::vector<std::vector<int2>>& per) {
  std::vector<int> key;
  for (const auto& l : per) {
    key.push_back((int)l.size());
    for (const int2& jb : l) {
      key.push_back(jb.x);
      key.push_back(jb.y);
    }
  }
  if (!P->waves.empty() && key == P->wave_key) return;
  GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));  // no launch still reads the old job lists
  std::vector<std::vector<int4>> small, big;
  std::vector<int> ptr(1, 0);
  int pos = 0;
  for (int n = 0; n < (int)per.size(); ++n) {
    std::map<int, int> last_write, last_read;
    for (const int2& jb : per[n]) {
      const VDesc& d = P->vd[jb.x];
      const int de = d.out_de[jb.y];
      int l = 0;
      for (int p = 0; p < d.k; ++p) {
        if (p == jb.y) continue;
        auto w = last_write.find(d.in_de[p]);
        if (w != last_write.end()) l = std::max(l, w->second + 1);
      }
      auto r = last_read.find(de);
      if (r != last_read.end()) l = std::max(l, r->second + 1);
      auto w = last_write.find(de);
      if (w != last_write.end()) l = std::max(l, w->second + 1);
      last_write[de] = l;
      last_read.erase(de);
      for (int p = 0; p < d.k; ++p) {
        if (p == jb.y) continue;
        int& lr = last_read.emplace(d.in_de[p], l).first->second;
        lr = std::max(lr, l);
      }
      auto& lv = d.n <= kSmallN ? small : big;
      if ((int)lv.size() <= l) {
        small.resize(l + 1);
        big.resize(l + 1);
      }
      (d.n <= kSmallN ? small : big)[l].push_back(make_int4(jb.x, jb.y, pos, n));
      ++pos;
    }
    ptr.push_back(pos);
  }
  std::vector<int4> all;
  std::vector<std::pair<size_t, int>> spans;  // (offset, count) per wave and class
  for (size_t l = 0; l < small.size(); ++l)
    for (auto* lv : {&small[l], &big[l]}) {
      spans.push_back({all.size(), (int)lv->size()});
      all.insert(all.end(), lv->begin(), lv->end());
    }
  if (all.empty()) all.push_back(make_int4(0, 0, 0, 0));
  P->d_wave_jobs.upload(all, P->ctx->stream);
  P->d_wave_ptr.upload(ptr, P->ctx->stream);
  std::vector<int> iota(std::max(pos, 1));
  std::iota(iota.begin(), iota.end(), 0);
  P->d_wave_iota.upload(iota, P->ctx->stream);
  P->d_pos_diffs.alloc(std::max(pos, 1));
  P->waves.clear();
  for (size_t l = 0; l < small.size(); ++l) {
    std::pair<WaveJobs, WaveJobs> w;
    for (int c = 0; c < 2; ++c) {
      WaveJobs& j = c == 0 ? w.first : w.second;
      const auto& sp = spans[2 * l + c];
      j.d_jobs = P->d_wave_jobs.p + sp.first;
      j.count = sp.second;
      j.team = c == 0 ? 32 : 256;
      for (const int4& jb : c == 0 ? small[l] : big[l]) j.ncap = std::max(j.ncap, P->vd[jb.x].n);
    }
    P->waves.push_back(w);
  }
  P->wave_key = key;
  P->wave_version++;
  P->clear_graphs();
}

// Sweeps of the sequential schedule as waves (see build_waves), in place on
// msgs, in arithmetic `arith`; per-network convergence as the other schedules.
// Sequential sweeps in waves: `maxiter` sweeps in arithmetic `arith`, per-network
// convergence at `tol` (< 0: none), and a reduced-precision phase's noise-floor
// stop after `stall` sweeps without progress (0: none).
void run_waves(gbtn_plan* P, int arith, const void* fac, const void* bra, void* msgs, int maxiter, double tol,
               int normalize, int stall = 0) {
  cudaStream_t s = P->ctx->stream;
  const bool want_diff = tol >= 0.0;
  GBTN_CUDA(cudaMemsetAsync(P->d_conv.p, 0, sizeof(int) * P->nnet, s));
  GBTN_CUDA(cudaMemsetAsync(P->d_iters.p, 0, sizeof(int) * P->nnet, s));
  GBTN_CUDA(cudaMemsetAsync(P->d_nconv.p, 0, sizeof(int), s));
  const int* conv = want_diff ? P->d_conv.p : nullptr;
  const GraphKey key{20 + arith, GBTN_SCHED_SEQUENTIAL, normalize, want_diff ? 1 : 0, stall, P->wave_version,
                     P->list_version, tol};
  sweep_loop(P, maxiter, key, [&] {
    for (const auto& w : P->waves) {
      launch_bp_wave_any(arith, w.first, P->d_vd.p, fac, bra, msgs, P->d_msg_off.p, P->d_pos_diffs.p, conv,
                         normalize, want_diff, s);
      launch_bp_wave_any(arith, w.second, P->d_vd.p, fac, bra, msgs, P->d_msg_off.p, P->d_pos_diffs.p, conv,
                         normalize, want_diff, s);
    }
    if (want_diff)
      launch_reduce_diffs(P->nnet, P->d_wave_ptr.p, P->d_wave_iota.p, P->d_pos_diffs.p, tol, P->d_conv.p,
                          P->d_iters.p, P->d_mean.p, s, stall, P->d_best.p, P->d_since.p, P->d_nconv.p);
  }, want_diff);
}

// The sequential schedule of a plan that holds large vertices: every message
// of the sequence in order through the global-memory path (one vertex at a
// time, each update seeing every earlier one, in place), FP64 or FP32 (complex
// ones too); per sweep the mean diff of each network's sequence is tested on
// the host (abstractbeliefpropagationcache.jl:272-287, 313-329).  Latency-bound:
// a few launches per message.
void run_sequential_large(gbtn_plan* P, const gbtn_bp_opts* o, const std::vector<std::vector<int2>>& per,
                          int32_t* iters, double* mean_diff) {
  cudaStream_t s = P->ctx->stream;
  const bool want_diff = o->tol >= 0.0;
  const bool f32 = o->precision == GBTN_F32;
  const int arith = P->cplx ? (f32 ? kArithZ32 : kArithZ64) : (f32 ? kArithF32 : kArithF64);
  const void* fac = P->d_fac.p;
  const void* bra = P->sep_bra ? P->d_bra.p : nullptr;
  void* msgs = P->d_msg[P->cur].p;
  if (f32) {
    ensure_f32(P);
    launch_convert_f64_to_f32(P->d_msg[P->cur].p, P->d_msg32[0].p, P->es() * P->n_msg, s);
    fac = P->d_fac32.p;
    bra = P->sep_bra ? P->d_bra32.p : nullptr;
    msgs = P->d_msg32[0].p;
  }
  std::vector<int> it(P->nnet, 0);
  std::vector<double> md(P->nnet, NAN);
  std::vector<char> done(P->nnet, 0);
  std::vector<double> diffs(2 * (size_t)P->ne);
  for (int sweep = 1; sweep <= o->maxiter; ++sweep) {
    bool any = false;
    for (int n = 0; n < P->nnet; ++n) {
      if (done[n]) continue;
      any = true;
      for (const int2& e : per[n]) large_one_message(P, arith, e.x, e.y, fac, bra, msgs, msgs, o->normalize,
                                                     want_diff ? 1 : 0, s);
      it[n] = sweep;
    }
    if (!any) break;
    if (!want_diff) continue;
    GBTN_CUDA(cudaMemcpyAsync(diffs.data(), P->d_diffs.p, sizeof(double) * diffs.size(), cudaMemcpyDeviceToHost, s));
    GBTN_CUDA(cudaStreamSynchronize(s));
    for (int n = 0; n < P->nnet; ++n) {
      if (done[n]) continue;
      double sum = 0.0;
      for (const int2& e : per[n]) sum += diffs[P->vd[e.x].out_de[e.y]];
      md[n] = sum / (double)per[n].size();
      if (md[n] <= o->tol) done[n] = 1;
    }
  }
  if (f32) launch_convert_f32_to_f64(P->d_msg32[0].p, P->d_msg[P->cur].p, P->es() * P->n_msg, s);
  GBTN_CUDA(cudaStreamSynchronize(s));
  if (iters) std::copy(it.begin(), it.end(), iters);
  if (mean_diff) std::copy(md.begin(), md.end(), mean_diff);
}

void compute_rdms(gbtn_plan* P) {
  cudaStream_t s = P->ctx->stream;
  if (P->cplx) {
    for (const WorkList* wl : {&P->lists[0].first, &P->lists[0].second})
      launch_vertex_rdms<zdouble>(*wl, P->d_vd.p, zptr(P->d_fac.p), P->sep_bra ? zptr(P->d_bra.p) : nullptr,
                                  zptr(P->d_msg[P->cur].p), P->d_msg_off.p, P->d_rdm_off.p, zptr(P->d_rdm.p), s);
    large_rdms(P, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr, P->d_msg[P->cur].p, P->d_rdm.p);
    return;
  }
  // real plans: the contractions in double-FP32 (~48-bit, FP64 in and out),
  // at ~2.7x the FP64 pipe's rate; traces, ratios and logs stay FP64
  for (const WorkList* wl : {&P->lists[0].first, &P->lists[0].second})
    launch_vertex_rdms_df32(*wl, P->d_vd.p, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr, P->d_msg[P->cur].p,
                            P->d_msg_off.p, P->d_rdm_off.p, P->d_rdm.p, s);
  large_rdms(P, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr, P->d_msg[P->cur].p, P->d_rdm.p);
}

}  // namespace

// Small kernels of the API layer.
__global__ void expect1_kernel(int nv, const long long* rdm_off, const double* rdm, const int* dsite, const double* ops,
                               const long long* op_off, double* out) {
  const int v = blockIdx.x * blockDim.x + threadIdx.x;
  if (v >= nv) return;
  const int d = dsite[v];
  const double* r = rdm + rdm_off[v];
  const double* o = ops + (op_off ? op_off[v] : 0);
  double num = 0.0, den = 0.0;
  for (int i = 0; i < d * d; ++i) num += r[i] * o[i];
  for (int q = 0; q < d; ++q) den += r[q + d * q];
  out[v] = num / den;
}

// rho[(s'u, s'v), (su, sv)] = sum_{b,a} Ru[s'u, su, b, a] Rv[s'v, sv, b, a]
// (the shared link's bra and ket indices contracted directly, no conjugation)
__device__ __forceinline__ double rdm_mac(double a, double b, double c) { return fma(a, b, c); }
__device__ __forceinline__ zdouble rdm_mac(zdouble a, zdouble b, zdouble c) {
  return zdouble(fma(a.re, b.re, fma(-a.im, b.im, c.re)), fma(a.re, b.im, fma(a.im, b.re, c.im)));
}
template <typename T>
__global__ void edge_rdm_combine_kernel(int nedges, const int* du_, const int* dv_, const int* chi_,
                                        const long long* hu_off, const long long* hv_off, const T* halves,
                                        const long long* out_off, T* out) {
  const int j = blockIdx.x;
  if (j >= nedges) return;
  const int du = du_[j], dv = dv_[j], c2 = chi_[j] * chi_[j];
  const int D = du * dv;
  for (int idx = threadIdx.x; idx < D * D; idx += blockDim.x) {
    const int row = idx % D, col = idx / D;
    const int spu = row % du, spv = row / du, su = col % du, sv = col / du;
    const T* ru = halves + hu_off[j] + (long long)(spu + du * su) * c2;
    const T* rv = halves + hv_off[j] + (long long)(spv + dv * sv) * c2;
    T acc = T(0.0);
    for (int i = 0; i < c2; ++i) acc = rdm_mac(ru[i], rv[i], acc);
    out[out_off[j] + idx] = acc;
  }
}

// Complex two-site RDMs (interleaved pairs): the real part of
// sum rho O / tr rho for a real operator O.
__global__ void expect2_z_kernel(int nedges, const long long* rdm_off, const int* D_, const zdouble* rdm,
                                 const double* op, double* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nedges) return;
  const int D = D_[j];
  const zdouble* r = rdm + rdm_off[j];
  double nr = 0.0, ni = 0.0, dr = 0.0, di = 0.0;
  for (int i = 0; i < D * D; ++i) {
    nr += r[i].re * op[i];
    ni += r[i].im * op[i];
  }
  for (int q = 0; q < D; ++q) {
    dr += r[q + D * q].re;
    di += r[q + D * q].im;
  }
  out[j] = (nr * dr + ni * di) / (dr * dr + di * di);
}

__global__ void expect2_kernel(int nedges, const long long* rdm_off, const int* D_, const double* rdm, const double* op,
                               double* out) {
  const int j = blockIdx.x * blockDim.x + threadIdx.x;
  if (j >= nedges) return;
  const int D = D_[j];
  const double* r = rdm + rdm_off[j];
  double num = 0.0, den = 0.0;
  for (int i = 0; i < D * D; ++i) num += r[i] * op[i];
  for (int q = 0; q < D; ++q) den += r[q + D * q];
  out[j] = num / den;
}

// Partition scale factors (rescale_partitions): ket *= vn/|ket|, bra *= s*vn/|bra|
// with Z' = Z/(|ket||bra|), s = sign(Z'), vn = |Z'|^(-1/2).  With a shared
// bra a negative Z' cannot be represented and yields NaN scales.
__global__ void partition_scale_kernel(int nv, const VDesc* vd, const double* fac, const double* bra,
                                       const long long* rdm_off, const double* rdm, double* scale) {
  const int v = blockIdx.x;
  const long long off = vd[v].a_off;
  const int n = vd[v].n, d = vd[v].d;
  double nk = 0.0, nb = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    nk += fac[off + i] * fac[off + i];
    if (bra) nb += bra[off + i] * bra[off + i];
  }
  __shared__ double r1[32], r2[32];
  for (int o = 16; o > 0; o >>= 1) {
    nk += __shfl_xor_sync(0xffffffffu, nk, o);
    nb += __shfl_xor_sync(0xffffffffu, nb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r1[threadIdx.x >> 5] = nk;
    r2[threadIdx.x >> 5] = nb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += r1[w];
      b += r2[w];
    }
    const double normk = sqrt(a);
    const double normb = bra ? sqrt(b) : normk;
    double z = 0.0;
    for (int q = 0; q < d; ++q) z += rdm[rdm_off[v] + q + d * q];
    const double zp = z / (normk * normb);
    const double sgn = zp > 0.0 ? 1.0 : (zp < 0.0 ? -1.0 : 0.0);
    const double vn = 1.0 / sqrt(fabs(zp));
    if (bra) {
      scale[2 * v] = vn / normk;
      scale[2 * v + 1] = sgn * vn / normb;
    } else {
      scale[2 * v] = sgn > 0.0 ? vn / normk : NAN;
      scale[2 * v + 1] = 1.0;
    }
  }
}

// Complex partition scale factors (abstractbeliefpropagationcache.jl:349-379).
// With z' = Z / (|ket| |bra|), r = z'^(-1/2) (principal root) and s = sign(z')
// when z' has an exactly zero imaginary part, else 1, the reference weights the
// first vertex of the partition by s * (s * r) and the others by s * r.  The
// partition lists the bra first (the form network is the disjoint union of
// operator, bra and ket, formnetworks/bilinearformnetwork.jl:34-38), so the ket
// takes s * r and the bra s * s * r; the stored bra is conjugated by every
// contraction, so it is scaled by the conjugate.  With a shared bra only the
// ket is scaled: the returned ket is the reference's and the partition scalar
// becomes z'/|z'| (1 for the real positive scalars of <psi|psi>).  scale: four
// doubles per vertex, (ket re, ket im, bra re, bra im), norms divided in.
// fac, bra: interleaved (re, im) doubles; rdm_off in complex elements.
__global__ void partition_scale_z_kernel(int nv, const VDesc* vd, const double* fac, const double* bra,
                                         const long long* rdm_off, const double* rdm, double* scale) {
  const int v = blockIdx.x;
  const long long off = 2 * vd[v].a_off;
  const int n = 2 * vd[v].n, d = vd[v].d;
  double nk = 0.0, nb = 0.0;
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    nk += fac[off + i] * fac[off + i];
    if (bra) nb += bra[off + i] * bra[off + i];
  }
  __shared__ double r1[32], r2[32];
  for (int o = 16; o > 0; o >>= 1) {
    nk += __shfl_xor_sync(0xffffffffu, nk, o);
    nb += __shfl_xor_sync(0xffffffffu, nb, o);
  }
  if ((threadIdx.x & 31) == 0) {
    r1[threadIdx.x >> 5] = nk;
    r2[threadIdx.x >> 5] = nb;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    double a = 0.0, b = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
      a += r1[w];
      b += r2[w];
    }
    const double normk = sqrt(a);
    const double normb = bra ? sqrt(b) : normk;
    double zr = 0.0, zi = 0.0;
    for (int q = 0; q < d; ++q) {
      zr += rdm[2 * (rdm_off[v] + q + d * q)];
      zi += rdm[2 * (rdm_off[v] + q + d * q) + 1];
    }
    zr /= normk * normb;
    zi /= normk * normb;
    // principal square root w of z' (w.re >= 0; the branch cut on the negative
    // real axis follows the sign of the zero imaginary part), then r = 1 / w
    const double m = hypot(zr, zi);
    const double h = sqrt(0.5 * (m + fabs(zr)));
    double wr, wi;
    if (zr >= 0.0) {
      wr = h;
      wi = h > 0.0 ? zi / (2.0 * h) : 0.0;
    } else {
      wr = fabs(zi) / (2.0 * h);
      wi = copysign(h, zi);
    }
    const double w2 = wr * wr + wi * wi;
    const double rr = w2 > 0.0 ? wr / w2 : INFINITY, ri = w2 > 0.0 ? -wi / w2 : 0.0;
    const double sg = zi == 0.0 ? (zr > 0.0 ? 1.0 : (zr < 0.0 ? -1.0 : 0.0)) : 1.0;
    scale[4 * v] = sg * rr / normk;
    scale[4 * v + 1] = sg * ri / normk;
    if (bra) {
      scale[4 * v + 2] = sg * sg * rr / normb;
      scale[4 * v + 3] = -sg * sg * ri / normb;
    } else {
      scale[4 * v + 2] = 1.0;
      scale[4 * v + 3] = 0.0;
    }
  }
}

// fac_v *= (scale[4v], scale[4v+1]), bra_v *= (scale[4v+2], scale[4v+3]) in
// complex arithmetic (interleaved (re, im) doubles).
__global__ void scale_vertices_z_kernel(int nv, const VDesc* vd, double* fac, double* bra, const double* scale) {
  const int v = blockIdx.x;
  if (v >= nv) return;
  const long long off = 2 * vd[v].a_off;
  const int n = vd[v].n;
  const double kr = scale[4 * v], ki = scale[4 * v + 1], br = scale[4 * v + 2], bi = scale[4 * v + 3];
  for (int i = threadIdx.x; i < n; i += blockDim.x) {
    const double x = fac[off + 2 * i], y = fac[off + 2 * i + 1];
    fac[off + 2 * i] = x * kr - y * ki;
    fac[off + 2 * i + 1] = x * ki + y * kr;
    if (bra) {
      const double p = bra[off + 2 * i], q = bra[off + 2 * i + 1];
      bra[off + 2 * i] = p * br - q * bi;
      bra[off + 2 * i + 1] = p * bi + q * br;
    }
  }
}

// m_de *= (f[2 de], f[2 de + 1]) in complex arithmetic, one block per directed edge.
__global__ void scale_messages_z_kernel(int nde, const int* dchi, const long long* msg_off, const double* f,
                                        double* msgs) {
  const int de = blockIdx.x;
  if (de >= nde) return;
  const double fr = f[2 * de], fi = f[2 * de + 1];
  if (fr == 1.0 && fi == 0.0) return;
  const int chi = dchi[de];  // per directed edge
  for (int i = threadIdx.x; i < chi * chi; i += blockDim.x) {
    const long long k = 2 * (msg_off[de] + i);
    const double x = msgs[k], y = msgs[k + 1];
    msgs[k] = x * fr - y * fi;
    msgs[k + 1] = x * fi + y * fr;
  }
}

namespace {

// Complex plans with bra = conj(ket): after the kets are scaled, partition v's
// scalar is z_v = e^{i phi_v} (the reference reaches 1 by scaling its bra with
// the unconjugated factor, which a shared bra cannot take).  Every message
// carries a free phase, and m_{u->v} *= e^{i psi}, m_{v->u} *= e^{-i psi}
// keeps every edge scalar <m_e, m_ebar> while it multiplies z_v by e^{i psi}
// and z_u by e^{-i psi}.  psi set on the edges of a breadth-first spanning
// forest, children before parents, brings every z_v to 1 but the roots'.
// Each root keeps the phase of the product of its component's z_v: 1 up to
// rounding when the component's BP estimate of <psi|psi> (invariant under
// message phases) is real and positive.
void move_partition_phases(gbtn_plan* P) {
  constexpr double kTwoPi = 6.283185307179586;
  cudaStream_t s = P->ctx->stream;
  compute_rdms(P);
  std::vector<double> r(2 * P->n_rdm);
  copy_out(P, r.data(), P->d_rdm.p, sizeof(double) * 2 * P->n_rdm, GBTN_HOST);
  std::vector<double> phi(P->nv);
  for (int v = 0; v < P->nv; ++v) {
    double zr = 0.0, zi = 0.0;
    for (int q = 0; q < P->dsite[v]; ++q) {
      zr += r[2 * (P->rdm_off[v] + q + P->dsite[v] * q)];
      zi += r[2 * (P->rdm_off[v] + q + P->dsite[v] * q) + 1];
    }
    if (!std::isfinite(zr) || !std::isfinite(zi) || (zr == 0.0 && zi == 0.0)) return;  // nothing to move
    phi[v] = std::atan2(zi, zr);
  }
  std::vector<std::vector<int>> adj(P->nv);
  for (int e = 0; e < P->ne; ++e) {
    adj[P->eu[e]].push_back(e);
    adj[P->ev[e]].push_back(e);
  }
  std::vector<int> order, parent(P->nv, -1);
  std::vector<char> seen(P->nv, 0);
  order.reserve(P->nv);
  for (int root = 0; root < P->nv; ++root) {
    if (seen[root]) continue;
    seen[root] = 1;
    size_t head = order.size();
    order.push_back(root);
    while (head < order.size()) {
      const int v = order[head++];
      for (int e : adj[v]) {
        const int w = P->eu[e] == v ? P->ev[e] : P->eu[e];
        if (seen[w]) continue;
        seen[w] = 1;
        parent[w] = e;
        order.push_back(w);
      }
    }
  }
  std::vector<double> acc(P->nv, 0.0), f(4 * (size_t)P->ne);
  for (int de = 0; de < 2 * P->ne; ++de) {
    f[2 * de] = 1.0;
    f[2 * de + 1] = 0.0;
  }
  for (int k = (int)order.size() - 1; k >= 0; --k) {
    const int v = order[k], e = parent[v];
    if (e < 0) continue;
    const int p = P->eu[e] == v ? P->ev[e] : P->eu[e];
    const double ps = std::remainder(-phi[v] - acc[v], kTwoPi);  // onto m_{p->v}; -ps onto m_{v->p}
    const int de_in = P->eu[e] == p ? 2 * e : 2 * e + 1;
    f[2 * de_in] = std::cos(ps);
    f[2 * de_in + 1] = std::sin(ps);
    f[2 * (de_in ^ 1)] = std::cos(ps);
    f[2 * (de_in ^ 1) + 1] = -std::sin(ps);
    acc[p] -= ps;
  }
  DevBuf<double> d_f;
  d_f.upload(f, s);
  scale_messages_z_kernel<<<2 * P->ne, 64, 0, s>>>(2 * P->ne, P->d_dchi.p, P->d_msg_off.p, d_f.p,
                                                   P->d_msg[P->cur].p);
  GBTN_CUDA(cudaGetLastError());
  GBTN_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

namespace gbtn {
cudaStream_t ctx_stream(gbtn_ctx* c) { return c->stream; }
void set_ctx_error(gbtn_ctx* c, const char* msg) { set_err(c, msg); }
}  // namespace gbtn

extern "C" {

int gbtn_abi_version(void) { return GBTN_ABI_VERSION; }

const char* gbtn_last_error(const gbtn_ctx* ctx) { return ctx ? ctx->err.c_str() : g_err_noctx.c_str(); }

int gbtn_ctx_create(int device, gbtn_ctx** out) {
  API_TRY
  require(out != nullptr, "out is NULL");
  *out = nullptr;
  int ndev = 0;
  GBTN_CUDA(cudaGetDeviceCount(&ndev));
  require(device >= 0 && device < ndev, "device index out of range");
  GBTN_CUDA(cudaSetDevice(device));
  auto c = std::make_unique<gbtn_ctx>();
  c->device = device;
  GBTN_CUDA(cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking));
  c->stream = c->own;
  c->sched = build_schedules();
  upload_schedules(c->sched);
  *out = c.release();
  API_CATCH(nullptr)
}

int gbtn_ctx_destroy(gbtn_ctx* ctx) {
  if (!ctx) return GBTN_OK;
  cudaSetDevice(ctx->device);
  if (ctx->own) {
    cudaStreamSynchronize(ctx->own);
    cudaStreamDestroy(ctx->own);
  }
  delete ctx;
  return GBTN_OK;
}

int gbtn_ctx_set_stream(gbtn_ctx* ctx, void* stream) {
  if (!ctx) return GBTN_ERR_INVALID;
  ctx->stream = stream ? reinterpret_cast<cudaStream_t>(stream) : ctx->own;
  return GBTN_OK;
}

void* gbtn_ctx_get_stream(const gbtn_ctx* ctx) { return ctx ? reinterpret_cast<void*>(ctx->stream) : nullptr; }

int gbtn_ctx_set_profiling(gbtn_ctx* ctx, int on) {
  if (!ctx) return GBTN_ERR_INVALID;
  ctx->profiling = on ? 1 : 0;
  return GBTN_OK;
}

int gbtn_ctx_test_wait_timeout(gbtn_ctx* ctx, int on) {
  gbtn_ctx* C = ctx;
  API_TRY
  require(ctx, "NULL context");
  gbtn::tc_set_test_extra_tx(on ? 16u : 0u);
  API_CATCH(C)
}

int gbtn_ctx_kernel_time(gbtn_ctx* ctx, int kernel_class, double* total_ms, int64_t* launches) {
  API_TRY
  require(ctx && total_ms && launches, "NULL argument");
  double ms = 0.0;
  int64_t n = 0;
  std::vector<gbtn_ctx::Rec> keep;
  for (auto& r : ctx->recs) {
    if (r.cls != kernel_class) {
      keep.push_back(r);
      continue;
    }
    GBTN_CUDA(cudaEventSynchronize(r.b));
    float t = 0.f;
    GBTN_CUDA(cudaEventElapsedTime(&t, r.a, r.b));
    ms += t;
    ++n;
    cudaEventDestroy(r.a);
    cudaEventDestroy(r.b);
  }
  ctx->recs.swap(keep);
  *total_ms = ms;
  *launches = n;
  API_CATCH(ctx)
}

int gbtn_plan_create(gbtn_ctx* ctx, const gbtn_graph_desc* g, gbtn_plan** out) {
  API_TRY
  require(ctx && g && out, "NULL argument");
  *out = nullptr;
  GBTN_CUDA(cudaSetDevice(ctx->device));
  require(g->nv >= 1 && g->ne >= 0, "graph needs nv >= 1 and ne >= 0");
  require(g->ne == 0 || (g->edge_u && g->edge_v && g->edge_dim), "edge arrays are NULL");
  require(g->site_dim && g->leg_ptr && (g->leg_edge || g->ne == 0), "vertex arrays are NULL");
  auto P = std::make_unique<gbtn_plan>();
  P->ctx = ctx;
  P->nv = g->nv;
  P->ne = g->ne;
  P->sep_bra = g->separate_bra != 0;
  P->cplx = g->complex_values != 0;
  P->nnet = g->vertex_network ? g->n_networks : 1;
  require(P->nnet >= 1, "n_networks must be >= 1");
  P->eu.assign(g->edge_u, g->edge_u + g->ne);
  P->ev.assign(g->edge_v, g->edge_v + g->ne);
  P->dsite.assign(g->site_dim, g->site_dim + g->nv);
  P->vnet.assign(g->nv, 0);
  if (g->vertex_network) P->vnet.assign(g->vertex_network, g->vertex_network + g->nv);
  for (int v = 0; v < g->nv; ++v) {
    require(P->vnet[v] >= 0 && P->vnet[v] < P->nnet, "vertex_network out of range");
    require(P->dsite[v] >= 1, "site dimension must be >= 1");
    if (P->dsite[v] > kMaxSiteLarge) throw Unsupported("site dimension must be in 1..64");
  }
  P->dchi.resize(2 * (size_t)g->ne);
  for (int e = 0; e < g->ne; ++e) {
    const int u = P->eu[e], v = P->ev[e], c = g->edge_dim[e];
    require(u >= 0 && u < g->nv && v >= 0 && v < g->nv, "edge endpoint out of range");
    require(u != v, "self loops are not allowed");
    require(P->vnet[u] == P->vnet[v], "edge joins two different networks");
    require(c >= 1, "bond dimension must be >= 1");
    if (c > kMaxChiLarge) throw Unsupported("bond dimension must be in 1..64");
    P->dchi[2 * e] = P->dchi[2 * e + 1] = c;
  }
  // messages
  P->msg_off.resize(2 * (size_t)g->ne);
  long long off = 0;
  for (int de = 0; de < 2 * g->ne; ++de) {
    P->msg_off[de] = off;
    off += (long long)P->dchi[de] * P->dchi[de];
  }
  P->n_msg = off;
  // vertices
  require(g->leg_ptr[0] == 0, "leg_ptr[0] must be 0");
  std::vector<int> seen_count(g->ne, 0);
  P->vd.resize(g->nv);
  P->is_large.assign(g->nv, 0);
  off = 0;
  long long roff = 0;
  P->rdm_off.resize(g->nv);
  for (int v = 0; v < g->nv; ++v) {
    VDesc d{};
    const int b = g->leg_ptr[v], e_ = g->leg_ptr[v + 1];
    require(e_ >= b, "leg_ptr must be non-decreasing");
    d.k = e_ - b;
    if (d.k > kMaxDeg) throw Unsupported("vertex degree above 8");
    d.d = P->dsite[v];
    d.net = P->vnet[v];
    d.a_off = off;
    long long n = d.d;
    for (int p = 0; p < d.k; ++p) {
      const int e = g->leg_edge[b + p];
      require(e >= 0 && e < g->ne, "leg_edge out of range");
      require(P->eu[e] == v || P->ev[e] == v, "leg_edge names an edge not incident to the vertex");
      seen_count[e]++;
      d.chi[p] = P->dchi[2 * e];
      d.st[p] = (int)n;
      n *= d.chi[p];
      const bool fwd = P->eu[e] == v;
      d.out_de[p] = fwd ? 2 * e : 2 * e + 1;
      d.in_de[p] = fwd ? 2 * e + 1 : 2 * e;
    }
    if (n > kMaxLargeN) throw Unsupported("vertex tensor above 2^28 elements");
    d.n = (int)n;
    P->vd[v] = d;
    off += n;
    P->rdm_off[v] = roff;
    roff += (long long)d.d * d.d;
    P->maxdeg = std::max(P->maxdeg, d.k);
    // the shared-memory kernels hold the whole tensor (FP64 or complex FP64,
    // three or four buffers) and bond / site dimensions <= 8; the rest runs
    // the global-memory path
    bool large = d.d > kMaxSite || n > (1 << 20);
    for (int p = 0; p < d.k; ++p) large = large || d.chi[p] > kMaxChi;
    if (!large) {
      const int team = n <= kSmallN ? 32 : 256;
      const size_t need = smem_need((int)n, d.k, P->sep_bra, P->cplx ? sizeof(zdouble) : sizeof(double), team) *
                          (team == 32 ? 4 : 1);
      large = need > 227 * 1024;
    }
    P->is_large[v] = large ? 1 : 0;
    P->has_large = P->has_large || large;
    if (!large) P->ncap = std::max(P->ncap, (int)n);
  }
  for (int e = 0; e < g->ne; ++e) require(seen_count[e] == 2, "every edge must appear once in the legs of each endpoint");
  P->n_fac = off;
  P->n_rdm = roff;

  cudaStream_t s = ctx->stream;
  P->d_vd.upload(P->vd, s);
  P->d_msg_off.upload(P->msg_off, s);
  P->d_rdm_off.upload(P->rdm_off, s);
  P->d_dchi.upload(P->dchi, s);
  P->d_dsite.upload(P->dsite, s);
  const int es = P->es();
  P->d_fac.alloc(es * P->n_fac);
  GBTN_CUDA(cudaMemsetAsync(P->d_fac.p, 0, sizeof(double) * es * std::max<long long>(P->n_fac, 1), s));
  if (P->sep_bra) P->d_bra.alloc(es * P->n_fac);
  P->d_msg[0].alloc(es * std::max<long long>(P->n_msg, 1));
  P->d_msg[1].alloc(es * std::max<long long>(P->n_msg, 1));
  P->d_diffs.alloc(std::max<long long>(2LL * P->ne, 1));
  GBTN_CUDA(cudaMemsetAsync(P->d_diffs.p, 0xff, sizeof(double) * std::max<long long>(2LL * P->ne, 1),
                            P->ctx->stream));  // NaN until a sweep with a tolerance runs
  P->d_mean.alloc(P->nnet);
  P->d_conv.alloc(P->nnet);
  P->d_nconv.alloc(1);
  GBTN_CUDA(cudaMallocHost(&P->h_nconv, 2 * sizeof(int)));
  for (cudaEvent_t& e : P->poll_ev) GBTN_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  P->d_iters.alloc(P->nnet);
  P->d_phase_iters.alloc(4 * (size_t)P->nnet);
  GBTN_CUDA(cudaMemsetAsync(P->d_phase_iters.p, 0, sizeof(int) * 4 * P->nnet, s));
  P->d_since.alloc(P->nnet);
  P->d_best.alloc(P->nnet);
  P->d_rdm.alloc(es * std::max<long long>(P->n_rdm, 1));
  P->d_edge_sc.alloc(es * std::max(P->ne, 1));
  P->d_re.alloc(P->nnet);
  P->d_im.alloc(P->nnet);
  P->d_scale.alloc(2 * es * (size_t)P->nv);  // (ket, bra) factors per vertex, complex for complex plans

  // per-network bookkeeping (parallel-sequence order of directed edges)
  std::vector<std::vector<int>> nde(P->nnet), nvv(P->nnet), nee(P->nnet);
  for (int e = 0; e < g->ne; ++e) nde[P->vnet[P->eu[e]]].push_back(2 * e);
  for (int e = 0; e < g->ne; ++e) nde[P->vnet[P->eu[e]]].push_back(2 * e + 1);
  for (int v = 0; v < g->nv; ++v) nvv[P->vnet[v]].push_back(v);
  for (int e = 0; e < g->ne; ++e) nee[P->vnet[P->eu[e]]].push_back(e);
  auto csr = [&](const std::vector<std::vector<int>>& L, DevBuf<int>& ptr, DevBuf<int>& idx) {
    std::vector<int> p(1, 0), x;
    for (auto& l : L) {
      x.insert(x.end(), l.begin(), l.end());
      p.push_back((int)x.size());
    }
    ptr.upload(p, s);
    if (x.empty()) x.push_back(0);
    idx.upload(x, s);
  };
  csr(nde, P->d_net_de_ptr, P->d_net_de);
  csr(nvv, P->d_net_v_ptr, P->d_net_v);
  csr(nee, P->d_net_e_ptr, P->d_net_e);

  // work lists: all vertices, then greedy colour classes in vertex order
  std::vector<int> all(g->nv);
  std::iota(all.begin(), all.end(), 0);
  P->lists.push_back(split_list(P.get(), all));
  P->large_lists.push_back(build_large_waves(P.get(), all));
  P->d_iota.upload(all, s);
  P->d_zero_off.upload(std::vector<long long>(1, 0), s);
  if (P->has_large) reserve_single_vertex(P.get());
  std::vector<std::vector<int>> nbrs(g->nv);
  for (int e = 0; e < g->ne; ++e) {
    nbrs[P->eu[e]].push_back(P->ev[e]);
    nbrs[P->ev[e]].push_back(P->eu[e]);
  }
  P->color.assign(g->nv, -1);
  int ncol = 0;
  for (int v = 0; v < g->nv; ++v) {
    std::vector<char> used(g->nv + 1, 0);
    for (int w : nbrs[v])
      if (P->color[w] >= 0) used[P->color[w]] = 1;
    int c = 0;
    while (used[c]) ++c;
    P->color[v] = c;
    ncol = std::max(ncol, c + 1);
  }
  for (int c = 0; c < ncol; ++c) {
    std::vector<int> vs;
    for (int v = 0; v < g->nv; ++v)
      if (P->color[v] == c) vs.push_back(v);
    P->lists.push_back(split_list(P.get(), vs));
    P->large_lists.push_back(build_large_waves(P.get(), vs));
  }
  // tensor-core candidates: one swizzled BF16 image slot each; until the
  // first reduced-precision run tunes the split, only native vertices use it
  P->ncol = ncol;
  P->tc_cand.assign(g->nv, 0);
  if (!P->sep_bra && !P->cplx && P->n_msg < (1LL << 31))
    for (int v = 0; v < g->nv; ++v) P->tc_cand[v] = tc_paddable(P->vd[v]) ? 1 : 0;
  build_tc_slots(P.get());
  P->d_err.alloc(1);
  GBTN_CUDA(cudaMemsetAsync(P->d_err.p, 0, sizeof(int), s));
  {
    std::vector<char> use(g->nv, 0);
    for (int v = 0; v < g->nv; ++v) use[v] = P->tc_cand[v] && tc_native(P->vd[v]);
    build_tc_lists(P.get(), use);
  }
  launch_fill_messages(2 * P->ne, P->d_dchi.p, P->d_msg_off.p, P->d_msg[0].p, GBTN_INIT_IDENTITY, s, P->cplx);
  GBTN_CUDA(cudaStreamSynchronize(s));
  *out = P.release();
  API_CATCH(ctx)
}

int gbtn_plan_destroy(gbtn_plan* plan) {
  if (!plan) return GBTN_OK;
  cudaStreamSynchronize(plan->ctx->stream);
  delete plan;
  return GBTN_OK;
}

int gbtn_plan_sizes(const gbtn_plan* P, int64_t* n_factor, int64_t* n_message) {
  if (!P) return GBTN_ERR_INVALID;
  if (n_factor) *n_factor = P->n_fac;
  if (n_message) *n_message = P->n_msg;
  return GBTN_OK;
}

// Host -> device factor upload in kUploadChunks vertex ranges on a copy
// stream; the BF16 images of each range's tensor-core slots are built on a
// second stream as soon as the range has landed, so the builds hide under the
// copy (which the host link bounds).  Slots follow vertex order, so a vertex
// range owns a contiguous slot range.  Ends synchronised, like every HOST copy.
void upload_with_images(gbtn_plan* P, const double* ket) {
  cudaStream_t s = P->ctx->stream;
  if (!P->up_copy) {
    GBTN_CUDA(cudaStreamCreateWithFlags(&P->up_copy, cudaStreamNonBlocking));
    GBTN_CUDA(cudaStreamCreateWithFlags(&P->up_build, cudaStreamNonBlocking));
    for (cudaEvent_t& e : P->up_ev) GBTN_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
  }
  // both side streams start after the work already queued on the plan's stream
  GBTN_CUDA(cudaEventRecord(P->up_ev[kUploadChunks], s));
  GBTN_CUDA(cudaStreamWaitEvent(P->up_copy, P->up_ev[kUploadChunks], 0));
  GBTN_CUDA(cudaStreamWaitEvent(P->up_build, P->up_ev[kUploadChunks], 0));
  int slot = 0;
  for (int c = 0; c < kUploadChunks; ++c) {
    const int vb = (int)((long long)P->nv * c / kUploadChunks), ve = (int)((long long)P->nv * (c + 1) / kUploadChunks);
    const long long fb = vb < P->nv ? P->vd[vb].a_off : P->n_fac;
    const long long fe = ve < P->nv ? P->vd[ve].a_off : P->n_fac;
    if (fe > fb)
      GBTN_CUDA(cudaMemcpyAsync(P->d_fac.p + fb, ket + fb, sizeof(double) * (fe - fb), cudaMemcpyHostToDevice,
                                P->up_copy));
    GBTN_CUDA(cudaEventRecord(P->up_ev[c], P->up_copy));
    const int sb = slot;
    while (slot < (int)P->tc_slot_vertex.size() && P->tc_slot_vertex[slot] < ve) ++slot;
    if (slot > sb) {
      GBTN_CUDA(cudaStreamWaitEvent(P->up_build, P->up_ev[c], 0));
      launch_build_zimg(P->d_tc_slot_vertex.p + sb, slot - sb, P->d_vd.p, P->d_fac.p, P->d_zimg.p + (size_t)sb * 8192,
                        P->up_build);
    }
  }
  GBTN_CUDA(cudaEventRecord(P->up_ev[kUploadChunks], P->up_build));
  GBTN_CUDA(cudaStreamWaitEvent(s, P->up_ev[kUploadChunks], 0));
  GBTN_CUDA(cudaStreamWaitEvent(s, P->up_ev[kUploadChunks - 1], 0));
  GBTN_CUDA(cudaStreamSynchronize(s));
  P->zimg_valid = true;
}

int gbtn_set_factors(gbtn_plan* P, const double* ket, const double* bra, int mem) {
  const gbtn::NvtxRange nvtx_range("gbtn_set_factors");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && ket, "NULL argument");
  require(!P->sep_bra || bra, "plan has separate_bra: bra tensors are required");
  P->cnt_fac_up++;
  if (mem == GBTN_HOST && P->d_zimg.p && !P->cplx) {
    upload_with_images(P, ket);  // the plan has run BF16: rebuild its images while the factors arrive
  } else {
    copy_in(P, P->d_fac.p, ket, sizeof(double) * P->es() * P->n_fac, mem);
    P->zimg_valid = false;
  }
  if (P->sep_bra) copy_in(P, P->d_bra.p, bra, sizeof(double) * P->es() * P->n_fac, mem);
  P->fac32_valid = false;
  API_CATCH(C)
}

int gbtn_get_factors(gbtn_plan* P, double* ket, int mem) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && ket, "NULL argument");
  P->cnt_fac_down++;
  copy_out(P, ket, P->d_fac.p, sizeof(double) * P->es() * P->n_fac, mem);
  API_CATCH(C)
}

int gbtn_set_messages(gbtn_plan* P, const double* m, int mem) {
  const gbtn::NvtxRange nvtx_range("gbtn_set_messages");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && m, "NULL argument");
  P->cnt_msg_up++;
  copy_in(P, P->d_msg[P->cur].p, m, sizeof(double) * P->es() * P->n_msg, mem);
  API_CATCH(C)
}

int gbtn_get_messages(gbtn_plan* P, double* m, int mem) {
  const gbtn::NvtxRange nvtx_range("gbtn_get_messages");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && m, "NULL argument");
  P->cnt_msg_down++;
  copy_out(P, m, P->d_msg[P->cur].p, sizeof(double) * P->es() * P->n_msg, mem);
  API_CATCH(C)
}

int gbtn_get_edge_diffs(gbtn_plan* P, double* d, int mem) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && d, "NULL argument");
  copy_out(P, d, P->d_diffs.p, sizeof(double) * 2 * (size_t)P->ne, mem);
  API_CATCH(C)
}

int gbtn_init_messages(gbtn_plan* P, int kind) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL plan");
  require(kind == GBTN_INIT_IDENTITY || kind == GBTN_INIT_ONES, "unknown message init");
  launch_fill_messages(2 * P->ne, P->d_dchi.p, P->d_msg_off.p, P->d_msg[P->cur].p, kind, P->ctx->stream, P->cplx);
  API_CATCH(C)
}

int gbtn_bp_run(gbtn_plan* P, const gbtn_bp_opts* o, int32_t* iters, double* mean_diff) {
  const gbtn::NvtxRange nvtx_range("gbtn_bp_run");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && o, "NULL argument");
  require(o->maxiter >= 1, "You need to specify a number of iterations for BP!");
  require(o->schedule >= 0 && o->schedule <= 2, "unknown schedule");
  require(o->precision >= 0 && o->precision <= 4, "unknown precision");
  require(o->refine == GBTN_REFINE_DF32 || o->refine == GBTN_REFINE_F64, "unknown refinement arithmetic");
  require(o->confirm_f64 >= 0, "confirm_f64 must be >= 0");
  for (int& f : P->phase_fixed) f = 0;
  GBTN_CUDA(cudaMemsetAsync(P->d_phase_iters.p, 0, sizeof(int) * 4 * P->nnet, P->ctx->stream));
  cudaStream_t s = P->ctx->stream;
  const bool want_diff = o->tol >= 0.0;
  if (P->ne == 0) {
    finish_iters(P, false, o->maxiter, iters, mean_diff);
    return GBTN_OK;
  }
  if (o->precision == GBTN_BF16 && o->schedule == GBTN_SCHED_SEQUENTIAL)
    throw Unsupported("BF16 sweeps run the parallel or coloured schedule");
  if ((o->precision == GBTN_DF32 || o->precision == GBTN_MIXED) && o->schedule == GBTN_SCHED_SEQUENTIAL &&
      P->has_large)
    throw Unsupported("double-FP32 and mixed sequential sweeps take vertices of the shared-memory kernels only");
  if (P->cplx && o->precision == GBTN_BF16)
    throw Unsupported("complex tensors have no tensor-core (BF16) path: use f32, mixed or f64");
  if (P->cplx && o->precision == GBTN_DF32)
    throw Unsupported("complex tensors have no double-FP32 path: use f32, mixed or f64");
  // phase slots of gbtn_plan_phase_sweeps: 0 BF16, 1 FP32, 2 refinement, 3 FP64
  auto phase_done = [&](int slot, double phase_tol, int sweeps_run) {
    if (phase_tol >= 0.0)
      record_phase(P, slot);  // the reduction kernel counted each network's sweeps
    else
      P->phase_fixed[slot] = sweeps_run;  // no convergence test: every sweep ran
  };
  if (o->schedule == GBTN_SCHED_SEQUENTIAL) {
    require(o->edge_sequence && o->edge_sequence_len > 0, "SEQUENTIAL needs an edge sequence");
    std::vector<std::vector<int2>> per(P->nnet);
    for (int i = 0; i < o->edge_sequence_len; ++i) {
      const int de = o->edge_sequence[i];
      require(de >= 0 && de < 2 * P->ne, "edge_sequence entry out of range");
      const int e = de / 2;
      const int v = (de & 1) ? P->ev[e] : P->eu[e];
      int leg = -1;
      for (int p = 0; p < P->vd[v].k; ++p)
        if (P->vd[v].out_de[p] == de) leg = p;
      per[P->vnet[v]].push_back(make_int2(v, leg));
    }
    std::vector<int2> seq;
    std::vector<int> ptr(1, 0);
    for (auto& l : per) {
      require(!l.empty() || P->nnet == 1, "edge_sequence misses a network");
      seq.insert(seq.end(), l.begin(), l.end());
      ptr.push_back((int)seq.size());
    }
    for (int n = 0; n < P->nnet; ++n) require(ptr[n + 1] > ptr[n], "edge_sequence misses a network");
    if (P->has_large) {
      run_sequential_large(P, o, per, iters, mean_diff);
      return GBTN_OK;
    }
    // waves of independent messages, in sequence order (see build_waves)
    build_waves(P, per);
    const void* bra64 = P->sep_bra ? P->d_bra.p : nullptr;
    auto f32_waves = [&](int maxit, double tol, int stall) {
      ensure_f32(P);
      launch_convert_f64_to_f32(P->d_msg[P->cur].p, P->d_msg32[0].p, P->es() * P->n_msg, s);
      run_waves(P, P->cplx ? kArithZ32 : kArithF32, P->d_fac32.p, P->sep_bra ? P->d_bra32.p : nullptr,
                P->d_msg32[0].p, maxit, tol, o->normalize, stall);
      launch_convert_f32_to_f64(P->d_msg32[0].p, P->d_msg[P->cur].p, P->es() * P->n_msg, s);
    };
    if (o->precision == GBTN_F32) {
      f32_waves(o->maxiter, o->tol, 0);
      phase_done(1, o->tol, o->maxiter);
      finish_iters(P, want_diff, o->maxiter, iters, mean_diff);
    } else if (o->precision == GBTN_MIXED) {
      // FP32 waves to their tolerance or noise floor, then double-FP32 (or
      // FP64) waves to tol from that point; the BF16 tensor-core kernel
      // computes every message of a vertex at once, which this schedule's
      // one-message jobs do not use
      const double tol32 = o->tol_f32 > 0 ? o->tol_f32 : 1e-13;
      const int it32 = o->maxiter_f32 > 0 ? o->maxiter_f32 : o->maxiter;
      f32_waves(it32, tol32, kStallSweeps);
      phase_done(1, tol32, it32);
      const int nref = o->refine_f64 > 0 ? std::min(o->refine_f64, o->maxiter) : o->maxiter;
      const int arith = P->cplx ? kArithZ64 : (o->refine == GBTN_REFINE_F64 ? kArithF64 : kArithDF32);
      run_waves(P, arith, P->d_fac.p, bra64, P->d_msg[P->cur].p, nref, o->tol, o->normalize);
      phase_done(2, o->tol, nref);
      int last = nref;
      if (o->confirm_f64 > 0 && !P->cplx && arith == kArithDF32) {
        last = std::min(o->confirm_f64, o->maxiter);
        run_waves(P, kArithF64, P->d_fac.p, bra64, P->d_msg[P->cur].p, last, o->tol, o->normalize);
        phase_done(3, o->tol, last);
      }
      finish_iters(P, want_diff, last, iters, mean_diff);
    } else {
      const int arith = P->cplx ? kArithZ64 : (o->precision == GBTN_DF32 ? kArithDF32 : kArithF64);
      run_waves(P, arith, P->d_fac.p, bra64, P->d_msg[P->cur].p, o->maxiter, o->tol, o->normalize);
      phase_done(o->precision == GBTN_DF32 ? 2 : 3, o->tol, o->maxiter);
      finish_iters(P, want_diff, o->maxiter, iters, mean_diff);
    }
    return GBTN_OK;
  }
  if (P->cplx && o->precision == GBTN_F64) {
    run_sweeps<zdouble>(P, o->schedule, o->maxiter, o->tol, o->normalize, zptr(P->d_msg[0].p), zptr(P->d_msg[1].p),
                        zptr(P->d_fac.p), P->sep_bra ? zptr(P->d_bra.p) : nullptr, P->cur);
    phase_done(3, o->tol, o->maxiter);
    finish_iters(P, want_diff, o->maxiter, iters, mean_diff);
  } else if (P->cplx) {  // complex FP32 sweeps (F32), then FP64 ones (MIXED): no tensor-core phase
    ensure_f32(P);
    int c32 = 0;
    launch_convert_f64_to_f32(P->d_msg[P->cur].p, P->d_msg32[0].p, 2 * P->n_msg, s);
    const bool mixed = o->precision == GBTN_MIXED;
    const double tol32 = mixed ? (o->tol_f32 > 0 ? o->tol_f32 : 1e-13) : o->tol;
    const int it32 = mixed && o->maxiter_f32 > 0 ? o->maxiter_f32 : o->maxiter;
    run_sweeps<zfloat>(P, o->schedule, it32, tol32, o->normalize, zfptr(P->d_msg32[0].p), zfptr(P->d_msg32[1].p),
                       zfptr(P->d_fac32.p), P->sep_bra ? zfptr(P->d_bra32.p) : nullptr, c32,
                       mixed ? kStallSweeps : 0);
    phase_done(1, tol32, it32);
    launch_convert_f32_to_f64(P->d_msg32[c32].p, P->d_msg[P->cur].p, 2 * P->n_msg, s);
    if (mixed) {
      const int nref = o->refine_f64 > 0 ? std::min(o->refine_f64, o->maxiter) : o->maxiter;
      run_sweeps<zdouble>(P, o->schedule, nref, o->tol, o->normalize, zptr(P->d_msg[0].p), zptr(P->d_msg[1].p),
                          zptr(P->d_fac.p), P->sep_bra ? zptr(P->d_bra.p) : nullptr, P->cur);
      phase_done(2, o->tol, nref);
      finish_iters(P, want_diff, nref, iters, mean_diff);
    } else {
      finish_iters(P, want_diff, o->maxiter, iters, mean_diff);
    }
  } else if (o->precision == GBTN_F64) {
    run_sweeps<double>(P, o->schedule, o->maxiter, o->tol, o->normalize, P->d_msg[0].p, P->d_msg[1].p, P->d_fac.p,
                       P->sep_bra ? P->d_bra.p : nullptr, P->cur);
    phase_done(3, o->tol, o->maxiter);
    finish_iters(P, want_diff, o->maxiter, iters, mean_diff);
  } else if (o->precision == GBTN_DF32) {
    run_sweeps<double, DF32>(P, o->schedule, o->maxiter, o->tol, o->normalize, P->d_msg[0].p, P->d_msg[1].p,
                             P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr, P->cur);
    phase_done(2, o->tol, o->maxiter);
    finish_iters(P, want_diff, o->maxiter, iters, mean_diff);
  } else if (o->precision == GBTN_F32) {
    ensure_f32(P);
    int c32 = 0;
    launch_convert_f64_to_f32(P->d_msg[P->cur].p, P->d_msg32[0].p, P->n_msg, s);
    run_sweeps<float>(P, o->schedule, o->maxiter, o->tol, o->normalize, P->d_msg32[0].p, P->d_msg32[1].p, P->d_fac32.p,
                      P->sep_bra ? P->d_bra32.p : nullptr, c32);
    phase_done(1, o->tol, o->maxiter);
    launch_convert_f32_to_f64(P->d_msg32[c32].p, P->d_msg[P->cur].p, P->n_msg, s);
    finish_iters(P, want_diff, o->maxiter, iters, mean_diff);
  } else if (o->precision == GBTN_BF16) {
    ensure_f32_bufs(P);
    int c32 = 0;
    launch_convert_f64_to_f32(P->d_msg[P->cur].p, P->d_msg32[0].p, P->n_msg, s);
    tune_tc_split(P);
    if (bf16_has_simt(P)) ensure_f32(P);  // with every vertex on the tensor cores the FP32 factors go unread
    ensure_zimg(P);
    run_sweeps_bf16(P, o->schedule, o->maxiter, o->tol, o->normalize, c32);
    phase_done(0, o->tol, o->maxiter);
    launch_convert_f32_to_f64(P->d_msg32[c32].p, P->d_msg[P->cur].p, P->n_msg, s);
    finish_iters(P, want_diff, o->maxiter, iters, mean_diff);
  } else {  // MIXED: BF16 tensor-core phase, FP32 phase, then DF32 (or FP64) refinement
    ensure_f32(P);
    int c32 = 0;
    const double tol32 = o->tol_f32 > 0 ? o->tol_f32 : 1e-13;
    const int it32 = o->maxiter_f32 > 0 ? o->maxiter_f32 : o->maxiter;
    launch_convert_f64_to_f32(P->d_msg[P->cur].p, P->d_msg32[0].p, P->n_msg, s);
    if (o->schedule != GBTN_SCHED_SEQUENTIAL && !P->tc_slot_vertex.empty()) {
      tune_tc_split(P);
      ensure_zimg(P);
      const double tol16 = o->tol_bf16 > 0 ? o->tol_bf16 : 1e-6;
      const int it16 = o->maxiter_bf16 > 0 ? o->maxiter_bf16 : o->maxiter;
      run_sweeps_bf16(P, o->schedule, it16, tol16, o->normalize, c32, kStallSweeps);
      phase_done(0, tol16, it16);
    }
    run_sweeps<float>(P, o->schedule, it32, tol32, o->normalize, P->d_msg32[0].p, P->d_msg32[1].p, P->d_fac32.p,
                      P->sep_bra ? P->d_bra32.p : nullptr, c32, kStallSweeps);
    phase_done(1, tol32, it32);
    launch_convert_f32_to_f64(P->d_msg32[c32].p, P->d_msg[P->cur].p, P->n_msg, s);
    // refinement sweeps from the FP32 fixed point until tol (or refine_f64 / maxiter sweeps)
    const int nref = o->refine_f64 > 0 ? std::min(o->refine_f64, o->maxiter) : o->maxiter;
    if (o->refine == GBTN_REFINE_F64) {
      run_sweeps<double>(P, o->schedule, nref, o->tol, o->normalize, P->d_msg[0].p, P->d_msg[1].p, P->d_fac.p,
                         P->sep_bra ? P->d_bra.p : nullptr, P->cur);
      phase_done(2, o->tol, nref);
      finish_iters(P, want_diff, nref, iters, mean_diff);
    } else {
      run_sweeps<double, DF32>(P, o->schedule, nref, o->tol, o->normalize, P->d_msg[0].p, P->d_msg[1].p,
                               P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr, P->cur);
      phase_done(2, o->tol, nref);
      if (o->confirm_f64 > 0) {
        const int nc = std::min(o->confirm_f64, o->maxiter);
        run_sweeps<double>(P, o->schedule, nc, o->tol, o->normalize, P->d_msg[0].p, P->d_msg[1].p, P->d_fac.p,
                           P->sep_bra ? P->d_bra.p : nullptr, P->cur);
        phase_done(3, o->tol, nc);
        finish_iters(P, want_diff, nc, iters, mean_diff);
      } else {
        finish_iters(P, want_diff, nref, iters, mean_diff);
      }
    }
  }
  API_CATCH(C)
}

int gbtn_plan_counters(const gbtn_plan* P, int64_t* counts) {
  if (!P || !counts) return GBTN_ERR_INVALID;
  counts[0] = P->cnt_fac_up;
  counts[1] = P->cnt_msg_up;
  counts[2] = P->cnt_msg_down;
  counts[3] = P->cnt_fac_down;
  return GBTN_OK;
}

int gbtn_plan_phase_sweeps(gbtn_plan* P, int32_t* sweeps) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && sweeps, "NULL argument");
  std::vector<int> it(4 * (size_t)P->nnet);
  GBTN_CUDA(cudaMemcpyAsync(it.data(), P->d_phase_iters.p, sizeof(int) * it.size(), cudaMemcpyDeviceToHost,
                            P->ctx->stream));
  GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));
  for (int k = 0; k < 4; ++k) {
    int m = P->phase_fixed[k];
    for (int n = 0; n < P->nnet; ++n) m = std::max(m, it[(size_t)k * P->nnet + n]);
    sweeps[k] = m;
  }
  API_CATCH(C)
}

int gbtn_plan_set_tc_policy(gbtn_plan* P, int32_t policy) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL argument");
  require(policy >= GBTN_TC_AUTO && policy <= GBTN_TC_OFF, "unknown tensor-core policy");
  P->tc_policy = policy;
  P->tc_tuned = false;
  P->tc_tune_best_ms = 0.0;
  API_CATCH(C)
}

int gbtn_plan_set_graphs(gbtn_plan* P, int32_t on) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL argument");
  GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));
  if (!on) P->clear_graphs();
  P->graphs = on ? 1 : 0;
  API_CATCH(C)
}

int gbtn_plan_set_simt_tuning(gbtn_plan* P, int32_t on) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL argument");
  GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));
  require(on == 0 || on == 1 || on == 32 || on == 128 || on == 256, "SIMT tuning mode must be 0, 1, 32, 128 or 256");
  P->simt_tuning = on;
  for (int a = 0; a < 5; ++a) {
    P->team_tuned[a] = false;
    for (int k = 0; k < 32; ++k) P->team_pick[a][k] = 0;
  }
  ++P->list_version;
  API_CATCH(C)
}

int gbtn_plan_simt_teams(const gbtn_plan* P, int32_t arith, int32_t* teams) {
  if (!P || !teams || arith < 0 || arith > 4) return GBTN_ERR_INVALID;
  for (int k = 0; k < 32; ++k) teams[k] = P->team_pick[arith][k];
  return GBTN_OK;
}

int gbtn_plan_tc_split(gbtn_plan* P, int32_t* is_tc, double* tuned_ms) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && is_tc, "NULL argument");
  if (!P->tc_tuned) {
    ensure_f32(P);
    launch_convert_f64_to_f32(P->d_msg[P->cur].p, P->d_msg32[0].p, P->n_msg, P->ctx->stream);
    tune_tc_split(P);
  }
  for (int v = 0; v < P->nv; ++v) is_tc[v] = P->tc_use[v] ? 1 : 0;
  if (tuned_ms) *tuned_ms = P->tc_tune_best_ms;
  API_CATCH(C)
}

int gbtn_updated_message(gbtn_plan* P, int32_t de, double* out) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && out, "NULL argument");
  require(de >= 0 && de < 2 * P->ne, "directed edge out of range");
  const int e = de / 2;
  const int v = (de & 1) ? P->ev[e] : P->eu[e];
  int leg = -1;
  for (int p = 0; p < P->vd[v].k; ++p)
    if (P->vd[v].out_de[p] == de) leg = p;
  const int c = P->dchi[de];
  if (P->is_large[v]) {
    // global-memory path: the message lands at its own offset of a message-sized buffer
    DevBuf<double> tmp;
    tmp.alloc(P->es() * std::max<long long>(P->n_msg, 1));
    large_one_message(P, P->cplx ? kArithZ64 : kArithF64, v, leg, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr,
                      P->d_msg[P->cur].p, tmp.p, 1, 0, P->ctx->stream);
    copy_out(P, out, tmp.p + P->es() * P->msg_off[de], sizeof(double) * P->es() * c * c, GBTN_HOST);
    return GBTN_OK;
  }
  P->d_out.alloc(P->es() * c * c);
  if (P->cplx)
    launch_updated_message<zdouble>(P->d_vd.p, v, leg, zptr(P->d_fac.p), P->sep_bra ? zptr(P->d_bra.p) : nullptr,
                                    zptr(P->d_msg[P->cur].p), P->d_msg_off.p, zptr(P->d_out.p), P->ncap,
                                    P->ctx->stream);
  else
    launch_updated_message<double>(P->d_vd.p, v, leg, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr,
                                   P->d_msg[P->cur].p, P->d_msg_off.p, P->d_out.p, P->ncap, P->ctx->stream);
  copy_out(P, out, P->d_out.p, sizeof(double) * P->es() * c * c, GBTN_HOST);
  API_CATCH(C)
}

int gbtn_vertex_rdms(gbtn_plan* P, double* out) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && out, "NULL argument");
  compute_rdms(P);
  copy_out(P, out, P->d_rdm.p, sizeof(double) * P->es() * P->n_rdm, GBTN_HOST);
  API_CATCH(C)
}

int gbtn_expect1(gbtn_plan* P, const double* ops, int per_vertex, double* out) {
  const gbtn::NvtxRange nvtx_range("gbtn_expect1");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && ops && out, "NULL argument");
  cudaStream_t s = P->ctx->stream;
  compute_rdms(P);
  DevBuf<double> d_ops, d_res;
  DevBuf<long long> d_opoff;
  if (per_vertex) {
    std::vector<double> h(ops, ops + P->n_rdm);
    d_ops.upload(h, s);
    d_opoff.upload(P->rdm_off, s);
  } else {
    for (int v = 0; v < P->nv; ++v)
      require(P->dsite[v] == P->dsite[0], "a shared operator needs one site dimension; pass per-vertex operators");
    std::vector<double> h(ops, ops + P->dsite[0] * P->dsite[0]);
    d_ops.upload(h, s);
  }
  d_res.alloc(P->nv);
  if (P->cplx) {
    launch_expect1_z(P->nv, P->d_rdm_off.p, zptr(P->d_rdm.p), P->d_dsite.p, d_ops.p, per_vertex ? d_opoff.p : nullptr,
                     d_res.p, s);
  } else {
    expect1_kernel<<<(P->nv + 127) / 128, 128, 0, s>>>(P->nv, P->d_rdm_off.p, P->d_rdm.p, P->d_dsite.p, d_ops.p,
                                                        per_vertex ? d_opoff.p : nullptr, d_res.p);
    GBTN_CUDA(cudaGetLastError());
  }
  copy_out(P, out, d_res.p, sizeof(double) * P->nv, GBTN_HOST);
  API_CATCH(C)
}

static void edge_rdms_device(gbtn_plan* P, const int32_t* edges, int32_t n, DevBuf<double>& d_out,
                             std::vector<long long>& out_off) {
  cudaStream_t s = P->ctx->stream;
  std::vector<int> jobs;
  std::vector<long long> hoff;
  std::vector<int> du, dv, ch;
  std::vector<long long> hu, hv;
  long long off = 0, ooff = 0;
  out_off.clear();
  for (int j = 0; j < n; ++j) {
    const int e = edges[j];
    require(e >= 0 && e < P->ne, "edge out of range");
    const int u = P->eu[e], v = P->ev[e];
    if (P->is_large[u] || P->is_large[v])
      throw Unsupported("two-site RDMs are computed for vertices of the shared-memory kernels only "
                        "(bond and site dimensions <= 8)");
    int pu = -1, pv = -1;
    for (int p = 0; p < P->vd[u].k; ++p)
      if (P->vd[u].out_de[p] == 2 * e) pu = p;
    for (int p = 0; p < P->vd[v].k; ++p)
      if (P->vd[v].out_de[p] == 2 * e + 1) pv = p;
    const int c = P->dchi[2 * e];
    jobs.push_back(u);
    jobs.push_back(pu);
    hoff.push_back(off);
    hu.push_back(off);
    off += (long long)P->dsite[u] * P->dsite[u] * c * c;
    jobs.push_back(v);
    jobs.push_back(pv);
    hoff.push_back(off);
    hv.push_back(off);
    off += (long long)P->dsite[v] * P->dsite[v] * c * c;
    du.push_back(P->dsite[u]);
    dv.push_back(P->dsite[v]);
    ch.push_back(c);
    out_off.push_back(ooff);
    const long long D = (long long)P->dsite[u] * P->dsite[v];
    ooff += D * D;
  }
  P->d_jobs.upload(jobs, s);
  P->d_half_off.upload(hoff, s);
  P->d_halves.alloc(std::max<long long>(P->es() * off, 1));
  if (P->cplx)
    launch_edge_halves<zdouble>(P->d_jobs.p, 2 * n, P->ncap, P->maxdeg, P->d_vd.p, zptr(P->d_fac.p),
                                P->sep_bra ? zptr(P->d_bra.p) : nullptr, zptr(P->d_msg[P->cur].p), P->d_msg_off.p,
                                zptr(P->d_halves.p), P->d_half_off.p, s);
  else
    launch_edge_halves<double>(P->d_jobs.p, 2 * n, P->ncap, P->maxdeg, P->d_vd.p, P->d_fac.p,
                               P->sep_bra ? P->d_bra.p : nullptr, P->d_msg[P->cur].p, P->d_msg_off.p, P->d_halves.p,
                               P->d_half_off.p, s);
  DevBuf<int> d_du, d_dv, d_ch;
  DevBuf<long long> d_hu, d_hv, d_oo;
  d_du.upload(du, s);
  d_dv.upload(dv, s);
  d_ch.upload(ch, s);
  d_hu.upload(hu, s);
  d_hv.upload(hv, s);
  d_oo.upload(out_off, s);
  d_out.alloc(std::max<long long>(P->es() * ooff, 1));
  if (P->cplx)
    edge_rdm_combine_kernel<zdouble><<<n, 128, 0, s>>>(n, d_du.p, d_dv.p, d_ch.p, d_hu.p, d_hv.p, zptr(P->d_halves.p),
                                                       d_oo.p, zptr(d_out.p));
  else
    edge_rdm_combine_kernel<double><<<n, 128, 0, s>>>(n, d_du.p, d_dv.p, d_ch.p, d_hu.p, d_hv.p, P->d_halves.p,
                                                      d_oo.p, d_out.p);
  GBTN_CUDA(cudaGetLastError());
  GBTN_CUDA(cudaStreamSynchronize(s));
}

int gbtn_edge_rdms(gbtn_plan* P, const int32_t* edges, int32_t n, double* out) {
  const gbtn::NvtxRange nvtx_range("gbtn_edge_rdms");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && edges && out && n >= 0, "bad argument");
  if (n == 0) return GBTN_OK;
  DevBuf<double> d_out;
  std::vector<long long> oo;
  edge_rdms_device(P, edges, n, d_out, oo);
  long long tot = 0;
  for (int j = 0; j < n; ++j) {
    const int e = edges[j];
    const long long D = (long long)P->dsite[P->eu[e]] * P->dsite[P->ev[e]];
    tot += D * D;
  }
  copy_out(P, out, d_out.p, sizeof(double) * P->es() * tot, GBTN_HOST);
  API_CATCH(C)
}

int gbtn_expect2(gbtn_plan* P, const int32_t* edges, int32_t n, const double* op, double* out) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && edges && op && out && n >= 0, "bad argument");
  if (n == 0) return GBTN_OK;
  cudaStream_t s = P->ctx->stream;
  std::vector<int> D(n);
  for (int j = 0; j < n; ++j) {
    const int e = edges[j];
    require(e >= 0 && e < P->ne, "edge out of range");
    D[j] = P->dsite[P->eu[e]] * P->dsite[P->ev[e]];
    require(D[j] == D[0], "a shared two-site operator needs equal site dimensions");
  }
  DevBuf<double> d_rdm, d_op, d_res;
  std::vector<long long> oo;
  edge_rdms_device(P, edges, n, d_rdm, oo);
  DevBuf<long long> d_oo;
  DevBuf<int> d_D;
  d_oo.upload(oo, s);
  d_D.upload(D, s);
  std::vector<double> hop(op, op + D[0] * D[0]);
  d_op.upload(hop, s);
  d_res.alloc(n);
  if (P->cplx)
    expect2_z_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, d_oo.p, d_D.p, zptr(d_rdm.p), d_op.p, d_res.p);
  else
    expect2_kernel<<<(n + 127) / 128, 128, 0, s>>>(n, d_oo.p, d_D.p, d_rdm.p, d_op.p, d_res.p);
  GBTN_CUDA(cudaGetLastError());
  copy_out(P, out, d_res.p, sizeof(double) * n, GBTN_HOST);
  API_CATCH(C)
}

int gbtn_vertex_scalars(gbtn_plan* P, double* out) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && out, "NULL argument");
  compute_rdms(P);
  const int es = P->es();
  std::vector<double> r(es * P->n_rdm);
  copy_out(P, r.data(), P->d_rdm.p, sizeof(double) * es * P->n_rdm, GBTN_HOST);
  // trace of each d x d block (a host-side read-out of the device RDMs);
  // complex plans write (re, im) pairs
  for (int v = 0; v < P->nv; ++v)
    for (int c = 0; c < es; ++c) {
      double z = 0.0;
      for (int q = 0; q < P->dsite[v]; ++q) z += r[es * (P->rdm_off[v] + q + P->dsite[v] * q) + c];
      out[es * v + c] = z;
    }
  API_CATCH(C)
}

int gbtn_edge_scalars(gbtn_plan* P, double* out) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && out, "NULL argument");
  if (P->ne == 0) return GBTN_OK;
  if (P->cplx)
    launch_edge_scalars_z(P->ne, P->d_dchi.p, P->d_msg_off.p, zptr(P->d_msg[P->cur].p), zptr(P->d_edge_sc.p),
                          P->ctx->stream);
  else
    launch_edge_scalars(P->ne, P->d_dchi.p, P->d_msg_off.p, P->d_msg[P->cur].p, P->d_edge_sc.p, P->ctx->stream);
  copy_out(P, out, P->d_edge_sc.p, sizeof(double) * P->es() * P->ne, GBTN_HOST);
  API_CATCH(C)
}

int gbtn_logscalar(gbtn_plan* P, double* re, double* im) {
  const gbtn::NvtxRange nvtx_range("gbtn_logscalar");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && re, "NULL argument");
  cudaStream_t s = P->ctx->stream;
  compute_rdms(P);
  if (P->cplx) {
    if (P->ne)
      launch_edge_scalars_z(P->ne, P->d_dchi.p, P->d_msg_off.p, zptr(P->d_msg[P->cur].p), zptr(P->d_edge_sc.p), s);
    launch_logscalar_z(P->nnet, P->d_net_v_ptr.p, P->d_net_v.p, P->d_net_e_ptr.p, P->d_net_e.p, P->d_rdm_off.p,
                       zptr(P->d_rdm.p), P->d_dsite.p, zptr(P->d_edge_sc.p), P->d_re.p, P->d_im.p, s);
    copy_out(P, re, P->d_re.p, sizeof(double) * P->nnet, GBTN_HOST);
    if (im) copy_out(P, im, P->d_im.p, sizeof(double) * P->nnet, GBTN_HOST);
    return GBTN_OK;
  }
  if (P->ne) launch_edge_scalars(P->ne, P->d_dchi.p, P->d_msg_off.p, P->d_msg[P->cur].p, P->d_edge_sc.p, s);
  launch_logscalar(P->nnet, P->d_net_v_ptr.p, P->d_net_v.p, P->d_net_e_ptr.p, P->d_net_e.p, P->d_rdm_off.p,
                   P->d_rdm.p, P->d_dsite.p, P->d_edge_sc.p, P->d_re.p, P->d_im.p, s);
  copy_out(P, re, P->d_re.p, sizeof(double) * P->nnet, GBTN_HOST);
  if (im) copy_out(P, im, P->d_im.p, sizeof(double) * P->nnet, GBTN_HOST);
  API_CATCH(C)
}

int gbtn_rescale_messages(gbtn_plan* P) {
  const gbtn::NvtxRange nvtx_range("gbtn_rescale_messages");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL plan");
  if (P->ne) {
    KTimer kt(P->ctx, GBTN_KCLASS_GAUGE);
    if (P->cplx)
      launch_rescale_messages_z(P->ne, P->d_dchi.p, P->d_msg_off.p, zptr(P->d_msg[P->cur].p), P->ctx->stream);
    else
      launch_rescale_messages(P->ne, P->d_dchi.p, P->d_msg_off.p, P->d_msg[P->cur].p, P->ctx->stream,
                              *std::max_element(P->dchi.begin(), P->dchi.end()));
  }
  GBTN_CUDA(cudaStreamSynchronize(P->ctx->stream));
  API_CATCH(C)
}

int gbtn_rescale_partitions(gbtn_plan* P) {
  const gbtn::NvtxRange nvtx_range("gbtn_rescale_partitions");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL plan");
  cudaStream_t s = P->ctx->stream;
  compute_rdms(P);
  if (P->cplx) {
    partition_scale_z_kernel<<<P->nv, 256, 0, s>>>(P->nv, P->d_vd.p, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr,
                                                    P->d_rdm_off.p, P->d_rdm.p, P->d_scale.p);
    GBTN_CUDA(cudaGetLastError());
    scale_vertices_z_kernel<<<P->nv, 256, 0, s>>>(P->nv, P->d_vd.p, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr,
                                                   P->d_scale.p);
    GBTN_CUDA(cudaGetLastError());
    P->fac32_valid = false;
    P->zimg_valid = false;
    if (!P->sep_bra && P->ne > 0) move_partition_phases(P);
    GBTN_CUDA(cudaStreamSynchronize(s));
    return GBTN_OK;
  }
  partition_scale_kernel<<<P->nv, 256, 0, s>>>(P->nv, P->d_vd.p, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr,
                                              P->d_rdm_off.p, P->d_rdm.p, P->d_scale.p);
  GBTN_CUDA(cudaGetLastError());
  launch_scale_vertices(P->nv, P->d_vd.p, P->d_fac.p, P->sep_bra ? P->d_bra.p : nullptr, P->d_scale.p, s);
  P->fac32_valid = false;
  P->zimg_valid = false;
  GBTN_CUDA(cudaStreamSynchronize(s));
  API_CATCH(C)
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Energies and gradients: chains of the adjoint kernels (adjoint.cu)
// ---------------------------------------------------------------------------
namespace {

struct Energy2 {
  gbtn_plan* P;
  int nterms = 0, d = 0;
  DevBuf<double> ops, coef, ket, t, Ee, scale, netE;
  std::vector<std::unique_ptr<DevBuf<double>>> F;  // F[0] identity term, F[k] term k
  DevBuf<int> allv;
};

// Unnormalised (or normalised) messages of every directed edge computed with
// ket tensor `ket` and bra = the plan's tensors (bra pointer NULL when ket is
// the plan's own tensors).
template <typename T>
void raw_forward_t(gbtn_plan* P, const double* ket, const double* bra, const double* msgs, double* out, int normalize) {
  cudaStream_t s = P->ctx->stream;
  launch_bp_vertices<T>(P->lists[0].first, P->d_vd.p, as<T>(ket), as<T>(bra), as<T>(msgs), as<T>(out),
                        P->d_msg_off.p, P->d_diffs.p, nullptr, normalize, 0, s);
  launch_bp_vertices<T>(P->lists[0].second, P->d_vd.p, as<T>(ket), as<T>(bra), as<T>(msgs), as<T>(out),
                        P->d_msg_off.p, P->d_diffs.p, nullptr, normalize, 0, s);
}

// (Complex plans: interleaved (re, im) doubles.)
void raw_forward(gbtn_plan* P, const double* ket, const double* bra, const double* msgs, double* out, int normalize) {
  if (P->cplx)
    raw_forward_t<zdouble>(P, ket, bra, msgs, out, normalize);
  else
    raw_forward_t<double>(P, ket, bra, msgs, out, normalize);
}

// (Complex plans: every buffer holds interleaved (re, im) doubles; the
// energy is the real part, its cotangents conj of the holomorphic derivatives.)
template <typename T>
const double* term_ket(Energy2& E, int k) {
  if (k == 0) return E.P->d_fac.p;
  const size_t es = sizeof(T) / sizeof(double);
  launch_site_op<T>(E.P->nv, E.P->d_vd.p, as<T>(E.P->d_fac.p), as<T>(E.ops.p + (size_t)(k - 1) * E.d * E.d * es),
                    as<T>(E.ket.p), E.P->ctx->stream);
  return E.ket.p;
}

void energy_setup(Energy2& E, gbtn_plan* P, int nterms, const double* coef, const double* ops) {
  require(!P->sep_bra, "energies and gradients need bra = conj(ket) (a quadratic-form network)");
  require(nterms >= 1 && coef && ops, "need at least one operator term");
  cudaStream_t s = P->ctx->stream;
  const size_t es = P->es();
  E.P = P;
  E.nterms = nterms;
  E.d = P->dsite[0];
  for (int v = 0; v < P->nv; ++v) require(P->dsite[v] == E.d, "all vertices must share the site dimension of the operators");
  const size_t need = vertex_vjp_smem(P->ncap, P->cplx ? sizeof(zdouble) : sizeof(double));
  if (need > 227 * 1024) throw Unsupported("vertex tensor too large for the adjoint kernels");
  std::vector<double> h(ops, ops + (size_t)nterms * E.d * E.d * es), c(coef, coef + nterms);
  E.ops.upload(h, s);
  E.coef.upload(c, s);
  E.ket.alloc(std::max<long long>(P->n_fac, 1) * es);
  E.t.alloc((size_t)(nterms + 1) * std::max(P->ne, 1) * es);
  E.scale.alloc((size_t)(nterms + 1) * std::max(P->ne, 1) * es);
  E.Ee.alloc(std::max(P->ne, 1));
  E.netE.alloc(P->nnet);
  for (int k = 0; k <= nterms; ++k) {
    E.F.push_back(std::make_unique<DevBuf<double>>());
    E.F.back()->alloc(std::max<long long>(P->n_msg, 1) * es);
  }
  std::vector<int> all(P->nv);
  std::iota(all.begin(), all.end(), 0);
  E.allv.upload(all, s);
}

// Forward energy at messages `msgs`: term messages, edge dots, per-edge energies
// and cotangent scales, per-network sums.
template <typename T>
void energy_forward_t(Energy2& E, const double* msgs) {
  gbtn_plan* P = E.P;
  cudaStream_t s = P->ctx->stream;
  const size_t es = sizeof(T) / sizeof(double);
  for (int k = 0; k <= E.nterms; ++k) {
    const double* ket = term_ket<T>(E, k);
    raw_forward(P, ket, k == 0 ? nullptr : P->d_fac.p, msgs, E.F[k]->p, 0);
    launch_edge_dot<T>(P->ne, P->d_dchi.p, P->d_msg_off.p, as<T>(E.F[k]->p),
                       as<T>(E.t.p + (size_t)k * P->ne * es), s);
  }
  launch_energy_terms<T>(P->ne, E.nterms, E.coef.p, as<T>(E.t.p), E.Ee.p, as<T>(E.scale.p), s);
  launch_net_sum(P->nnet, P->d_net_e_ptr.p, P->d_net_e.p, E.Ee.p, E.netE.p, s);
}

// Direct part of the energy gradient at messages `msgs`: g += dE/dm, grad += dE/dA.
template <typename T>
void energy_direct_vjp_t(Energy2& E, const double* msgs, double* cot, double* g, double* grad) {
  gbtn_plan* P = E.P;
  cudaStream_t s = P->ctx->stream;
  const size_t es = sizeof(T) / sizeof(double);
  for (int k = 0; k <= E.nterms; ++k) {
    launch_energy_cot<T>(2 * P->ne, P->d_dchi.p, P->d_msg_off.p, as<T>(E.F[k]->p),
                         as<T>(E.scale.p + (size_t)k * P->ne * es), as<T>(cot), s);
    const double* ket = term_ket<T>(E, k);
    launch_vertex_vjp<T>(E.allv.p, P->nv, P->d_vd.p, as<T>(ket), as<T>(P->d_fac.p), as<T>(msgs), as<T>(cot),
                         P->d_msg_off.p, k == 0 ? nullptr : as<T>(E.ops.p + (size_t)(k - 1) * E.d * E.d * es),
                         as<T>(g), as<T>(grad), P->ncap, s);
  }
}

void energy_forward(Energy2& E, const double* msgs) {
  if (E.P->cplx)
    energy_forward_t<zdouble>(E, msgs);
  else
    energy_forward_t<double>(E, msgs);
}

void energy_direct_vjp(Energy2& E, const double* msgs, double* cot, double* g, double* grad) {
  if (E.P->cplx)
    energy_direct_vjp_t<zdouble>(E, msgs, cot, g, grad);
  else
    energy_direct_vjp_t<double>(E, msgs, cot, g, grad);
}

// Backpropagation through T normalised Jacobi sweeps from identity messages,
// checkpointed every c sweeps; complex cotangents lose their message-phase
// components at every step (the energy is invariant under them).
template <typename T>
void unrolled_backward_t(gbtn_plan* P, const int* allv, int Tn, int c, std::vector<std::unique_ptr<DevBuf<double>>>& ck,
                         std::vector<std::unique_ptr<DevBuf<double>>>& seg, double* lam_p, double* dgrad, long long nm) {
  cudaStream_t s = P->ctx->stream;
  const int ndir = 2 * P->ne;
  DevBuf<double> fraw, fbar, mbar;
  fraw.alloc(nm);
  fbar.alloc(nm);
  mbar.alloc(nm);
  double* lam = lam_p;
  double* mb = mbar.p;
  for (int j = (Tn - 1) / c; j >= 0; --j) {
    const int t0 = j * c, t1 = std::min(Tn, (j + 1) * c);
    GBTN_CUDA(cudaMemcpyAsync(seg[0]->p, ck[j]->p, sizeof(double) * nm, cudaMemcpyDeviceToDevice, s));
    for (int i = 1; i < t1 - t0; ++i) raw_forward(P, P->d_fac.p, nullptr, seg[i - 1]->p, seg[i]->p, 1);
    for (int t = t1; t > t0; --t) {
      const double* mprev = seg[t - 1 - t0]->p;
      raw_forward(P, P->d_fac.p, nullptr, mprev, fraw.p, 0);
      launch_norm_vjp<T>(ndir, P->d_dchi.p, P->d_msg_off.p, as<T>(fraw.p), as<T>(lam), as<T>(fbar.p), s);
      GBTN_CUDA(cudaMemsetAsync(mb, 0, sizeof(double) * nm, s));
      launch_vertex_vjp<T>(allv, P->nv, P->d_vd.p, as<T>(P->d_fac.p), as<T>(P->d_fac.p), as<T>(mprev),
                           as<T>(fbar.p), P->d_msg_off.p, nullptr, as<T>(mb), as<T>(dgrad), P->ncap, s);
      if constexpr (std::is_same<T, zdouble>::value)
        launch_phase_project(ndir, P->d_dchi.p, P->d_msg_off.p, as<zdouble>(mprev), as<zdouble>(mb), s);
      std::swap(lam, mb);
    }
  }
}

// The unrolled computation: identity messages, T normalised Jacobi sweeps,
// every c-th kept in ck (ck[0] = identity, T/c + 1 of them), c segment
// buffers for the backward's recomputation; the final messages end in cur
// and in the plan.
struct Unrolled {
  std::vector<std::unique_ptr<DevBuf<double>>> ck, seg;
  DevBuf<double> cur, nxt;
  int T = 0, c = 1;
};

void unrolled_forward(gbtn_plan* P, int T, int checkpoint, long long nm, Unrolled& U) {
  cudaStream_t s = P->ctx->stream;
  U.T = T;
  U.c = checkpoint > 0 ? checkpoint : (int)std::ceil(std::sqrt((double)T));
  const int nck = T / U.c + 1;
  for (int j = 0; j < nck; ++j) {
    U.ck.push_back(std::make_unique<DevBuf<double>>());
    U.ck.back()->alloc(nm);
  }
  for (int j = 0; j < U.c; ++j) {
    U.seg.push_back(std::make_unique<DevBuf<double>>());
    U.seg.back()->alloc(nm);
  }
  U.cur.alloc(nm);
  U.nxt.alloc(nm);
  launch_fill_messages(2 * P->ne, P->d_dchi.p, P->d_msg_off.p, U.cur.p, GBTN_INIT_IDENTITY, s, P->cplx);
  GBTN_CUDA(cudaMemcpyAsync(U.ck[0]->p, U.cur.p, sizeof(double) * nm, cudaMemcpyDeviceToDevice, s));
  for (int t = 1; t <= T; ++t) {
    raw_forward(P, P->d_fac.p, nullptr, U.cur.p, U.nxt.p, 1);
    std::swap(U.cur.p, U.nxt.p);
    if (t % U.c == 0 && t / U.c < nck)
      GBTN_CUDA(cudaMemcpyAsync(U.ck[t / U.c]->p, U.cur.p, sizeof(double) * nm, cudaMemcpyDeviceToDevice, s));
  }
  GBTN_CUDA(cudaMemcpyAsync(P->d_msg[P->cur].p, U.cur.p, sizeof(double) * nm, cudaMemcpyDeviceToDevice, s));
}

// lam = dL/d(final messages) -> grad += dL/dA through the unrolled sweeps
// (complex: lam's message-phase components dropped first, as at every step).
void unrolled_backward(gbtn_plan* P, const int* allv, Unrolled& U, double* lam, double* dgrad, long long nm) {
  if (P->cplx) {
    launch_phase_project(2 * P->ne, P->d_dchi.p, P->d_msg_off.p, as<zdouble>(U.cur.p), as<zdouble>(lam),
                         P->ctx->stream);
    unrolled_backward_t<zdouble>(P, allv, U.T, U.c, U.ck, U.seg, lam, dgrad, nm);
  } else {
    unrolled_backward_t<double>(P, allv, U.T, U.c, U.ck, U.seg, lam, dgrad, nm);
  }
}

// lambda = g + (dF/dm)^T lambda at the fixed point `msgs`, then grad += (dF/dA)^T lambda
// (T = zdouble for complex plans: conjugate-transposed products, cotangents dL/dRe + i dL/dIm).
template <typename T>
void implicit_adjoint_t(gbtn_plan* P, const int* allv, const double* msgs_d, const double* g_d, double* grad_d,
                        int maxiter, double tol, int32_t* iters, double* resid) {
  constexpr bool cplx = std::is_same<T, zdouble>::value;
  cudaStream_t s = P->ctx->stream;
  const long long nm = std::max<long long>(P->n_msg, 1) * (long long)(sizeof(T) / sizeof(double));
  const int ndir = 2 * P->ne;
  const T* msgs = as<T>(msgs_d);
  T* grad = as<T>(grad_d);
  DevBuf<double> fraw, fbar, lam, lam2, mbar, acc, gp, lrot, rho;
  fraw.alloc(nm);
  fbar.alloc(nm);
  lam.alloc(nm);
  lam2.alloc(nm);
  mbar.alloc(nm);
  acc.alloc(2);
  raw_forward(P, P->d_fac.p, nullptr, msgs_d, fraw.p, 0);
  // complex: the cotangent without its message-phase components, and the phase
  // each message takes in one sweep (see edge_phase_kernel)
  const double* g0 = g_d;
  auto project = [&](double* x) {
    if constexpr (cplx) launch_phase_project(ndir, P->d_dchi.p, P->d_msg_off.p, msgs, as<zdouble>(x), s);
  };
  // the cotangent handed to the VJP of the update: R lam (complex), lam (real)
  auto rotated = [&](const double* x) -> const double* {
    if constexpr (cplx) {
      launch_edge_rotate(ndir, P->d_dchi.p, P->d_msg_off.p, as<zdouble>(rho.p), as<zdouble>(x), as<zdouble>(lrot.p),
                         s);
      return lrot.p;
    }
    return x;
  };
  if constexpr (cplx) {
    gp.alloc(nm);
    lrot.alloc(nm);
    rho.alloc(2 * (size_t)std::max(ndir, 1));
    launch_edge_phase(ndir, P->d_dchi.p, P->d_msg_off.p, msgs, as<zdouble>(fraw.p), as<zdouble>(rho.p), s);
    GBTN_CUDA(cudaMemcpyAsync(gp.p, g_d, sizeof(double) * nm, cudaMemcpyDeviceToDevice, s));
    project(gp.p);
    g0 = gp.p;
  }
  GBTN_CUDA(cudaMemcpyAsync(lam.p, g0, sizeof(double) * nm, cudaMemcpyDeviceToDevice, s));
  int it = 0;
  double rel = 0.0;
  for (it = 1; it <= maxiter; ++it) {
    launch_norm_vjp<T>(ndir, P->d_dchi.p, P->d_msg_off.p, as<T>(fraw.p), as<T>(rotated(lam.p)), as<T>(fbar.p), s);
    GBTN_CUDA(cudaMemsetAsync(mbar.p, 0, sizeof(double) * nm, s));
    launch_vertex_vjp<T>(allv, P->nv, P->d_vd.p, as<T>(P->d_fac.p), as<T>(P->d_fac.p), msgs, as<T>(fbar.p),
                         P->d_msg_off.p, nullptr, as<T>(mbar.p), nullptr, P->ncap, s);
    project(mbar.p);
    launch_axpy_resid(nm, g0, mbar.p, lam.p, lam2.p, acc.p, s);
    double h[2];
    GBTN_CUDA(cudaMemcpyAsync(h, acc.p, sizeof(h), cudaMemcpyDeviceToHost, s));
    GBTN_CUDA(cudaStreamSynchronize(s));
    std::swap(lam.p, lam2.p);
    rel = h[0] > 0.0 ? std::sqrt(h[1] / h[0]) : 0.0;
    if (!std::isfinite(rel)) throw CudaError("adjoint BP solve produced non-finite values");
    if (rel <= tol) break;
  }
  if (it > maxiter) it = maxiter;
  launch_norm_vjp<T>(ndir, P->d_dchi.p, P->d_msg_off.p, as<T>(fraw.p), as<T>(rotated(lam.p)), as<T>(fbar.p), s);
  launch_vertex_vjp<T>(allv, P->nv, P->d_vd.p, as<T>(P->d_fac.p), as<T>(P->d_fac.p), msgs, as<T>(fbar.p),
                       P->d_msg_off.p, nullptr, nullptr, grad, P->ncap, s);
  if (iters) *iters = it;
  if (resid) *resid = rel;
}

void implicit_adjoint(gbtn_plan* P, const int* allv, const double* msgs, const double* g, double* grad, int maxiter,
                      double tol, int32_t* iters, double* resid) {
  if (P->cplx)
    implicit_adjoint_t<zdouble>(P, allv, msgs, g, grad, maxiter, tol, iters, resid);
  else
    implicit_adjoint_t<double>(P, allv, msgs, g, grad, maxiter, tol, iters, resid);
}

}  // namespace

extern "C" {

int gbtn_energy2(gbtn_plan* P, int32_t nterms, const double* coef, const double* ops, double* energy) {
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL plan");
  if (P->has_large)
    throw Unsupported("energies and gradients take vertices of the shared-memory kernels only (bond and site "
                      "dimensions <= 8)");
  require(P && energy, "NULL argument");
  Energy2 E;
  energy_setup(E, P, nterms, coef, ops);
  energy_forward(E, P->d_msg[P->cur].p);
  copy_out(P, energy, E.netE.p, sizeof(double) * P->nnet, GBTN_HOST);
  API_CATCH(C)
}

int gbtn_energy2_grad(gbtn_plan* P, int32_t nterms, const double* coef, const double* ops, const gbtn_grad_opts* o,
                      double* energy, double* grad, int32_t* iters, double* resid) {
  const gbtn::NvtxRange nvtx_range("gbtn_energy2_grad");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL plan");
  if (P->has_large)
    throw Unsupported("energies and gradients take vertices of the shared-memory kernels only (bond and site "
                      "dimensions <= 8)");
  require(P && o && grad, "NULL argument");
  require(o->mode == GBTN_GRAD_IMPLICIT || o->mode == GBTN_GRAD_UNROLLED, "unknown gradient mode");
  cudaStream_t s = P->ctx->stream;
  Energy2 E;
  energy_setup(E, P, nterms, coef, ops);
  const long long es = P->es();
  const long long nm = std::max<long long>(P->n_msg, 1) * es, nf = std::max<long long>(P->n_fac, 1) * es;
  DevBuf<double> g, cot, dgrad;
  g.alloc(nm);
  cot.alloc(nm);
  dgrad.alloc(nf);
  GBTN_CUDA(cudaMemsetAsync(g.p, 0, sizeof(double) * nm, s));
  GBTN_CUDA(cudaMemsetAsync(dgrad.p, 0, sizeof(double) * nf, s));
  if (o->mode == GBTN_GRAD_IMPLICIT) {
    const double* m = P->d_msg[P->cur].p;
    energy_forward(E, m);
    energy_direct_vjp(E, m, cot.p, g.p, dgrad.p);
    implicit_adjoint(P, E.allv.p, m, g.p, dgrad.p, o->maxiter > 0 ? o->maxiter : 500, o->tol > 0 ? o->tol : 1e-12,
                     iters, resid);
  } else {
    const int T = o->unroll;
    require(T >= 1, "UNROLLED needs unroll >= 1");
    Unrolled U;
    unrolled_forward(P, T, o->checkpoint, nm, U);  // the final messages stay in the plan
    energy_forward(E, U.cur.p);
    energy_direct_vjp(E, U.cur.p, cot.p, g.p, dgrad.p);
    unrolled_backward(P, E.allv.p, U, g.p, dgrad.p, nm);
    if (iters) *iters = T;
    if (resid) *resid = 0.0;
  }
  if (energy) copy_out(P, energy, E.netE.p, sizeof(double) * P->nnet, GBTN_HOST);
  copy_out(P, grad, dgrad.p, sizeof(double) * P->n_fac * es, GBTN_HOST);
  API_CATCH(C)
}

}  // extern "C"

namespace {

// Checks shared by the scalar gradients (quadratic-form network, every
// vertex with a link, shared-memory vertices).
void scalar_grad_checks(gbtn_plan* P) {
  if (P->has_large)
    throw Unsupported("energies and gradients take vertices of the shared-memory kernels only (bond and site "
                      "dimensions <= 8)");
  require(!P->sep_bra, "gradients need bra = conj(ket) (a quadratic-form network)");
  for (int v = 0; v < P->nv; ++v)
    if (P->vd[v].k < 1) throw Unsupported("gradients take vertices with at least one link");
  if (vertex_vjp_smem(P->ncap, P->cplx ? sizeof(zdouble) : sizeof(double)) > 227 * 1024)
    throw Unsupported("vertex tensor too large for the adjoint kernels");
}

// Per-network sums of per-vertex (and, when ev is given, minus per-edge) values.
void net_sums(gbtn_plan* P, const DevBuf<double>& vv, const DevBuf<double>* ev, double* out) {
  std::vector<double> hv(P->nv), he(std::max(P->ne, 1));
  copy_out(P, hv.data(), vv.p, sizeof(double) * P->nv, GBTN_HOST);
  if (ev && P->ne) copy_out(P, he.data(), ev->p, sizeof(double) * P->ne, GBTN_HOST);
  std::vector<double> acc(P->nnet, 0.0);
  for (int v = 0; v < P->nv; ++v) acc[P->vnet[v]] += hv[v];
  if (ev)
    for (int e = 0; e < P->ne; ++e) acc[P->vnet[P->eu[e]]] -= he[e];
  std::copy(acc.begin(), acc.end(), out);
}

// The log-norm (mode 0) or one-site expectation (mode 1, operator `op`, d x d
// elements of T) and its gradient: direct cotangents of the vertex and edge
// terms, vertex VJPs, then the implicit adjoint through the fixed point.
template <typename T>
void scalar_grad_t(gbtn_plan* P, int mode, const double* op, const gbtn_grad_opts* o, double* value, double* grad,
                   int32_t* iters, double* resid) {
  cudaStream_t s = P->ctx->stream;
  const long long es = sizeof(T) / sizeof(double);
  const long long nm = std::max<long long>(P->n_msg, 1) * es, nf = std::max<long long>(P->n_fac, 1) * es;
  DevBuf<double> dop, ketO, F, FO, ci, co, g, dgrad, vval, eval;
  DevBuf<int> allv;
  std::vector<int> all(P->nv);
  std::iota(all.begin(), all.end(), 0);
  allv.upload(all, s);
  F.alloc(nm);
  ci.alloc(nm);
  g.alloc(nm);
  dgrad.alloc(nf);
  vval.alloc(P->nv);
  for (DevBuf<double>* b : {&ci, &g}) GBTN_CUDA(cudaMemsetAsync(b->p, 0, sizeof(double) * nm, s));
  GBTN_CUDA(cudaMemsetAsync(dgrad.p, 0, sizeof(double) * nf, s));
  const double* m = P->d_msg[P->cur].p;
  raw_forward(P, P->d_fac.p, nullptr, m, F.p, 0);
  if (mode == 0) {
    eval.alloc(std::max(P->ne, 1));
    launch_vertex_term_cot<T>(P->nv, P->d_vd.p, P->d_msg_off.p, as<T>(m), as<T>(F.p), nullptr, 0, as<T>(ci.p),
                              nullptr, as<T>(g.p), vval.p, s);
    launch_edge_term_cot<T>(P->ne, P->d_dchi.p, P->d_msg_off.p, as<T>(m), as<T>(g.p), eval.p, s);
    launch_vertex_vjp<T>(allv.p, P->nv, P->d_vd.p, as<T>(P->d_fac.p), as<T>(P->d_fac.p), as<T>(m), as<T>(ci.p),
                         P->d_msg_off.p, nullptr, as<T>(g.p), as<T>(dgrad.p), P->ncap, s);
  } else {
    const int d = P->dsite[0];
    dop.upload(std::vector<double>(op, op + (size_t)d * d * es), s);
    ketO.alloc(nf);
    FO.alloc(nm);
    co.alloc(nm);
    GBTN_CUDA(cudaMemsetAsync(co.p, 0, sizeof(double) * nm, s));
    launch_site_op<T>(P->nv, P->d_vd.p, as<T>(P->d_fac.p), as<T>(dop.p), as<T>(ketO.p), s);
    raw_forward(P, ketO.p, P->d_fac.p, m, FO.p, 0);
    launch_vertex_term_cot<T>(P->nv, P->d_vd.p, P->d_msg_off.p, as<T>(m), as<T>(F.p), as<T>(FO.p), 1, as<T>(ci.p),
                              as<T>(co.p), as<T>(g.p), vval.p, s);
    launch_vertex_vjp<T>(allv.p, P->nv, P->d_vd.p, as<T>(P->d_fac.p), as<T>(P->d_fac.p), as<T>(m), as<T>(ci.p),
                         P->d_msg_off.p, nullptr, as<T>(g.p), as<T>(dgrad.p), P->ncap, s);
    launch_vertex_vjp<T>(allv.p, P->nv, P->d_vd.p, as<T>(ketO.p), as<T>(P->d_fac.p), as<T>(m), as<T>(co.p),
                         P->d_msg_off.p, as<T>(dop.p), as<T>(g.p), as<T>(dgrad.p), P->ncap, s);
  }
  implicit_adjoint(P, allv.p, m, g.p, dgrad.p, o && o->maxiter > 0 ? o->maxiter : 500,
                   o && o->tol > 0 ? o->tol : 1e-12, iters, resid);
  copy_out(P, grad, dgrad.p, sizeof(double) * P->n_fac * es, GBTN_HOST);
  if (value) net_sums(P, vval, mode == 0 ? &eval : nullptr, value);
}

}  // namespace

extern "C" {

int gbtn_logscalar_grad(gbtn_plan* P, const gbtn_grad_opts* o, double* value, double* grad, int32_t* iters,
                        double* resid) {
  const gbtn::NvtxRange nvtx_range("gbtn_logscalar_grad");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && grad, "NULL argument");
  scalar_grad_checks(P);
  if (P->cplx)
    scalar_grad_t<zdouble>(P, 0, nullptr, o, value, grad, iters, resid);
  else
    scalar_grad_t<double>(P, 0, nullptr, o, value, grad, iters, resid);
  API_CATCH(C)
}

int gbtn_expect1_grad(gbtn_plan* P, const double* op, const gbtn_grad_opts* o, double* value, double* grad,
                      int32_t* iters, double* resid) {
  const gbtn::NvtxRange nvtx_range("gbtn_expect1_grad");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P && op && grad, "NULL argument");
  scalar_grad_checks(P);
  const int d = P->dsite[0];
  for (int v = 0; v < P->nv; ++v) require(P->dsite[v] == d, "all vertices must share the site dimension of the operator");
  if (P->cplx)
    scalar_grad_t<zdouble>(P, 1, op, o, value, grad, iters, resid);
  else
    scalar_grad_t<double>(P, 1, op, o, value, grad, iters, resid);
  API_CATCH(C)
}

int gbtn_bp_vjp(gbtn_plan* P, const double* msg_cot, const gbtn_grad_opts* o, double* grad, int32_t* iters,
                double* resid) {
  const gbtn::NvtxRange nvtx_range("gbtn_bp_vjp");
  gbtn_ctx* C = P ? P->ctx : nullptr;
  API_TRY
  require(P, "NULL plan");
  if (P->has_large)
    throw Unsupported("energies and gradients take vertices of the shared-memory kernels only (bond and site "
                      "dimensions <= 8)");
  require(P && msg_cot && o && grad, "NULL argument");
  require(o->mode == GBTN_GRAD_IMPLICIT || o->mode == GBTN_GRAD_UNROLLED, "unknown gradient mode");
  require(o->mode == GBTN_GRAD_IMPLICIT || o->unroll >= 1, "UNROLLED needs unroll >= 1");
  require(!P->sep_bra, "gradients need bra = conj(ket) (a quadratic-form network)");
  if (vertex_vjp_smem(P->ncap, P->cplx ? sizeof(zdouble) : sizeof(double)) > 227 * 1024)
    throw Unsupported("vertex tensor too large for the adjoint kernels");
  cudaStream_t s = P->ctx->stream;
  const long long es = P->es();
  const long long nm = std::max<long long>(P->n_msg, 1) * es, nf = std::max<long long>(P->n_fac, 1) * es;
  DevBuf<double> g, dgrad;
  DevBuf<int> allv;
  std::vector<double> hg(msg_cot, msg_cot + P->n_msg * es);
  hg.resize(nm, 0.0);
  g.upload(hg, s);
  dgrad.alloc(nf);
  GBTN_CUDA(cudaMemsetAsync(dgrad.p, 0, sizeof(double) * nf, s));
  std::vector<int> all(P->nv);
  std::iota(all.begin(), all.end(), 0);
  allv.upload(all, s);
  if (o->mode == GBTN_GRAD_IMPLICIT) {
    implicit_adjoint(P, allv.p, P->d_msg[P->cur].p, g.p, dgrad.p, o->maxiter > 0 ? o->maxiter : 500,
                     o->tol > 0 ? o->tol : 1e-12, iters, resid);
  } else {  // through `unroll` sweeps from identity messages, which stay in the plan
    Unrolled U;
    unrolled_forward(P, o->unroll, o->checkpoint, nm, U);
    unrolled_backward(P, allv.p, U, g.p, dgrad.p, nm);
    if (iters) *iters = o->unroll;
    if (resid) *resid = 0.0;
  }
  copy_out(P, grad, dgrad.p, sizeof(double) * P->n_fac * es, GBTN_HOST);
  API_CATCH(C)
}

}  // extern "C"
