// Internal declarations shared by the C-ABI layer and the kernels of libgbtn.
#pragma once

#include <cuda_runtime.h>
#include <cuda_bf16.h>
#include <stdint.h>

#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/gbtn.h"

#include <nvtx3/nvToolsExt.h>

namespace gbtn {

// NVTX range named after a C entry point, for profiler timelines (nsys, ncu
// NVTX filters); a no-op unless a profiling tool is attached.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

}  // namespace gbtn

namespace gbtn {

// Limits of the compiled kernels.
constexpr int kMaxDeg = 8;        // links per vertex (site index excluded)
constexpr int kMaxChi = 8;        // bond dimension per link
constexpr int kMaxSite = 8;       // physical dimension
constexpr int kMaxOps = 48;       // schedule length per degree
constexpr int kNumBufs = 4;       // shared-memory tensor buffers (0 = site tensor)

// Complex FP64 element, interleaved (re, im) like numpy complex128 and Julia
// ComplexF64; its arithmetic lives in bp_device.cuh.
struct __align__(16) zdouble {
  double re, im;
  zdouble() = default;
  __host__ __device__ constexpr zdouble(double r, double i = 0.0) : re(r), im(i) {}
};

// Complex FP32 element (the FP32 SIMT path of complex networks): interleaved
// (re, im) floats.
struct __align__(8) zfloat {
  float re, im;
  zfloat() = default;
  __host__ __device__ constexpr zfloat(float r, float i = 0.f) : re(r), im(i) {}
};

// Per-vertex descriptor, read by every message / environment kernel.
struct __align__(16) VDesc {
  long long a_off;          // element offset of the vertex tensor
  int n;                    // d * prod(chi)
  int d;                    // site dimension
  int k;                    // number of links
  int net;                  // network id
  int chi[kMaxDeg];         // bond dim of leg p
  int st[kMaxDeg];          // element stride of leg p (site stride is 1)
  int in_de[kMaxDeg];       // directed edge entering v on leg p
  int out_de[kMaxDeg];      // directed edge leaving v on leg p
};

// Shared-memory elements of a SIMT team beyond its tensor buffers: incoming
// messages (kMaxDeg x 64), the close reduction ((team / 32) x 64), close
// results (kMaxDeg x 64 for a team of several warps, else 64) and the
// previous outgoing messages (kMaxDeg x 64).
__host__ __device__ inline constexpr size_t team_tail_elems(int team) {
  return (size_t)kMaxDeg * 64 + (size_t)(team / 32) * 64 + (team > 32 ? (size_t)kMaxDeg * 64 : 64) +
         (size_t)kMaxDeg * 64;
}

// One step of a vertex schedule: ABSORB src->dst on leg, or CLOSE src on leg.
struct SchedOp {
  int8_t type;  // 0 absorb, 1 close
  int8_t src;
  int8_t dst;
  int8_t leg;
};

struct DeviceSched {
  SchedOp ops[kMaxDeg + 1][kMaxOps];
  int len[kMaxDeg + 1];
  int nbuf[kMaxDeg + 1];
};

// Build, for every degree, the shared-prefix schedule that produces all
// outgoing messages of a vertex (host side).
DeviceSched build_schedules();

struct CudaError : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct InvalidArg : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct Unsupported : std::runtime_error {
  using std::runtime_error::runtime_error;
};
struct Timeout : std::runtime_error {
  using std::runtime_error::runtime_error;
};

#define GBTN_CUDA(call)                                                             \
  do {                                                                              \
    cudaError_t err__ = (call);                                                     \
    if (err__ != cudaSuccess)                                                       \
      throw ::gbtn::CudaError(std::string(#call) + ": " + cudaGetErrorString(err__)); \
  } while (0)

// Launch parameters of a batch of vertices processed by one message kernel.
// The vertices are sorted by tensor size and cut into size classes (up to
// kMaxSub sub-ranges, one launch each), so that a class of small tensors gets
// shared memory, and resident blocks, for its own largest tensor only.
constexpr int kMaxSub = 8;
struct WorkList {
  int* d_vertices = nullptr;  // device list of vertex ids
  int count = 0;
  int ncap = 0;               // largest n in the list
  int maxdeg = 0;
  int team = 32;              // threads per vertex (32 or 256)
  int nsub = 0;               // size classes: [sub_begin[i], sub_begin[i] + sub_count[i])
  int sub_begin[kMaxSub] = {};
  int sub_count[kMaxSub] = {};
  int sub_ncap[kMaxSub] = {};
  int sub_maxdeg[kMaxSub] = {};
  // Measured team width per size class (host table indexed by class_key(ncap);
  // 0 or no table: the list's own team).
  const int* pick = nullptr;
  // The list restricted to size class i (the whole list when it has none),
  // with its measured team width when one was chosen.
  WorkList sub(int i) const {
    WorkList w = *this;
    w.nsub = 0;
    if (nsub != 0) {
      w.d_vertices = d_vertices + sub_begin[i];
      w.count = sub_count[i];
      w.ncap = sub_ncap[i];
      w.maxdeg = sub_maxdeg[i];
    }
    if (pick && pick[class_key(w.ncap)] != 0) w.team = pick[class_key(w.ncap)];
    return w;
  }
  // ceil(log2(n)): the size class a vertex count falls in (classes are powers of two)
  static int class_key(int n) {
    int k = 0;
    while ((1 << k) < n && k < 30) ++k;
    return k;
  }
  int nsubs() const { return nsub == 0 ? 1 : nsub; }
};

// Kernel launchers (bp_kernels.cu).  T = double, float, zdouble or zfloat.
template <typename T>
void launch_bp_vertices(const WorkList& wl, const VDesc* vd, const T* fac, const T* bra,
                        const T* msg_in, T* msg_out, const long long* msg_off, double* diffs,
                        const int* converged, int normalize, int want_diff, cudaStream_t s);

// Double-FP32 arithmetic (bp_device.cuh, df32) on FP64 tensors and messages.
void launch_bp_vertices_df32(const WorkList& wl, const VDesc* vd, const double* fac, const double* bra,
                             const double* msg_in, double* msg_out, const long long* msg_off, double* diffs,
                             const int* converged, int normalize, int want_diff, cudaStream_t s);

// Global-memory path for vertices beyond the shared-memory kernels
// (bp_large.cu): bond and site dimensions up to 64, tensors up to 2^28
// elements, intermediates in a scratch area in HBM, one launch per schedule
// step over a wave of vertices of one degree.
constexpr int kMaxChiLarge = 64;
constexpr int kMaxSiteLarge = 64;
constexpr long long kMaxLargeN = 1LL << 28;
constexpr int kTile = 4096;  // elements of one staged tile
// Arithmetic of a large-path launch (the storage is double, float, zdouble or
// zfloat; double under DF32).
enum { kArithF64 = 0, kArithF32 = 1, kArithDF32 = 2, kArithZ64 = 3, kArithZ32 = 4 };

// Tiles of the fibers of one leg (stride st, dimension chi) of a tensor of n
// elements: a tile covers leg indices [l0, l0 + Lt) of R consecutive outer
// rows (each st * chi elements), contiguous runs of memory of at most kTile.
struct LegTiling {
  int Lt, R, ntl, ntj;
  long long nouter;
};
__host__ __device__ inline LegTiling leg_tiling(int n, int st, int chi) {
  LegTiling g;
  const long long sc = (long long)st * chi;
  g.nouter = n / sc;
  if (sc <= kTile) {
    g.Lt = st;
    g.R = (int)(kTile / sc < g.nouter ? kTile / sc : g.nouter);
    g.ntl = 1;
    g.ntj = (int)((g.nouter + g.R - 1) / g.R);
  } else {
    const int lt = kTile / chi;
    g.Lt = lt < st ? lt : st;
    g.R = 1;
    g.ntl = (st + g.Lt - 1) / g.Lt;
    g.ntj = (int)g.nouter;
  }
  return g;
}

template <typename S>
struct LargeArgs {
  const int* verts;         // wave vertex ids
  const long long* buf_off; // element offset of each wave vertex's scratch buffers
  const VDesc* vd;
  const S* fac;
  const S* bra;             // NULL: bra = conj(fac)
  const S* msgs;            // incoming messages
  const long long* msg_off;
};
// One schedule step (ABSORB, or CLOSE + normalisation into msg_out) for a
// wave; msg_old is the message array of the previous values (message_diff).
void launch_large_op_any(int arith, const LargeArgs<double>& a, int nverts, int max_tiles, int max_chi,
                         const SchedOp& op, void* scratch, void* partial, long long vstride, const void* msg_old,
                         void* msg_out, double* diffs, const int* converged, int normalize, int want_diff,
                         cudaStream_t s);
// CLOSE on the site index of buffer src: rho_v[s', s] into rdm (FP64 or complex FP64).
void launch_large_rdm_any(int arith, const LargeArgs<double>& a, int nverts, int max_tiles, int src, void* scratch,
                          void* partial, long long vstride, void* rdm, const long long* rdm_off, cudaStream_t s);
size_t large_elem_size(int arith);

// Block-sparse networks (bp_kernels.cu): the share of every listed sector
// block in its outgoing messages (mode 0) or in rho_v (mode 1), unnormalised,
// into partial + part_off[slot]; the sums and normalisation are in bp_qn.cu.
void launch_qn_blocks(const WorkList& wl, const VDesc* bd, const double* blocks, const double* msg_in,
                      const long long* sec_off, double* partial, const long long* part_off, int mode,
                      cudaStream_t s);
// The same shares in FP32 (FP32 blocks, messages and shares) or in
// double-FP32 arithmetic on FP64 storage (mode 0: message shares).
void launch_qn_blocks_f32(const WorkList& wl, const VDesc* bd, const float* blocks, const float* msg_in,
                          const long long* sec_off, float* partial, const long long* part_off, cudaStream_t s);
void launch_qn_blocks_df32(const WorkList& wl, const VDesc* bd, const double* blocks, const double* msg_in,
                           const long long* sec_off, double* partial, const long long* part_off, cudaStream_t s);

// One wave of the sequential schedule (bp_kernels.cu): jobs (vertex, leg,
// sequence position, network), one message each, in place; team 32 (four jobs
// per block) or 256 threads per job, shared memory for tensors of ncap elements.
struct WaveJobs {
  const int4* d_jobs = nullptr;
  int count = 0;
  int team = 32;
  int ncap = 0;
};
void launch_bp_wave_any(int arith, const WaveJobs& wj, const VDesc* vd, const void* fac, const void* bra, void* msgs,
                        const long long* msg_off, double* pos_diffs, const int* converged, int normalize,
                        int want_diff, cudaStream_t s);


void launch_reduce_diffs(int n_networks, const int* net_de_ptr, const int* net_de, const double* diffs,
                         double tol, int* converged, int* iters, double* mean_diff, cudaStream_t s,
                         int stall = 0, double* best = nullptr, int* since = nullptr,
                         int* n_conv = nullptr);

template <typename T>
void launch_updated_message(const VDesc* vd, int v, int leg, const T* fac, const T* bra, const T* msgs,
                            const long long* msg_off, T* out, int ncap, cudaStream_t s);

template <typename T>
void launch_vertex_rdms(const WorkList& wl, const VDesc* vd, const T* fac, const T* bra,
                        const T* msgs, const long long* msg_off, const long long* rdm_off,
                        T* rdm, cudaStream_t s);
void launch_vertex_rdms_df32(const WorkList& wl, const VDesc* vd, const double* fac, const double* bra,
                             const double* msgs, const long long* msg_off, const long long* rdm_off, double* rdm,
                             cudaStream_t s);

template <typename T>
void launch_edge_halves(const int* jobs /*pairs (v, leg)*/, int njobs, int ncap, int maxdeg,
                        const VDesc* vd, const T* fac, const T* bra, const T* msgs,
                        const long long* msg_off, T* halves /* per job d*d*chi*chi */,
                        const long long* half_off, cudaStream_t s);

void launch_convert_f64_to_f32(const double* a, float* b, long long n, cudaStream_t s);
void launch_convert_f32_to_f64(const float* a, double* b, long long n, cudaStream_t s);
void launch_convert_f64_to_bf16(const double* a, __nv_bfloat16* b, long long n, cudaStream_t s);
void launch_fill_messages(int ndir, const int* dchi, const long long* msg_off, double* msgs, int kind,
                          cudaStream_t s,
                          int cplx = 0);
void launch_scale_vertices(int nv, const VDesc* vd, double* fac, double* bra, const double* scale,
                           cudaStream_t s);
void launch_rescale_messages_z(int ne, const int* dchi, const long long* msg_off, zdouble* msgs, cudaStream_t s);
void launch_rescale_messages(int ne, const int* dchi, const long long* msg_off, double* msgs,
                             cudaStream_t s, int max_chi = 8);
void launch_edge_scalars(int ne, const int* dchi, const long long* msg_off, const double* msgs,
                         double* out, cudaStream_t s);
void launch_logscalar(int n_networks, const int* net_v_ptr, const int* net_v, const int* net_e_ptr,
                      const int* net_e, const long long* rdm_off, const double* rdm, const int* dsite,
                      const double* edge_sc, double* re, double* im, cudaStream_t s);

// Complex plans: edge scalars sum m_e * m_ebar, log-scalar with principal
// complex logs, <O> from complex RDMs (real part, O real).
void launch_edge_scalars_z(int ne, const int* dchi, const long long* msg_off, const zdouble* msgs, zdouble* out,
                           cudaStream_t s);
void launch_logscalar_z(int n_networks, const int* net_v_ptr, const int* net_v, const int* net_e_ptr,
                        const int* net_e, const long long* rdm_off, const zdouble* rdm, const int* dsite,
                        const zdouble* edge_sc, double* re, double* im, cudaStream_t s);
void launch_expect1_z(int nv, const long long* rdm_off, const zdouble* rdm, const int* dsite, const double* ops,
                      const long long* op_off, double* out, cudaStream_t s);

// BF16 tensor-core path (bp_tc.cu): the kernel works on degree-4 vertices with
// d = 2 and chi = 8; a vertex with d = 2, at most four legs and chi <= 8 is
// zero-padded to that shape (missing legs carry the fixed 1 x 1 message 1).
// Per-vertex record (the kernel reads one per work item, in list order):
// element offsets of the incoming / outgoing messages on the four legs
// (compact chi x chi storage), the outgoing directed-edge ids (-1 on a padding
// leg), the network id, the four bond dimensions (one byte each, 0 on a
// padding leg) and the vertex's image slot.
struct __align__(16) TcRec {
  int in_off[4];
  int out_off[4];
  int out_de[4];
  int net;
  int chi4;
  int slot;  // image slot
  int pad;
};
bool tc_native(const VDesc& d);    // degree 4, d = 2, chi = 8 on every leg
bool tc_paddable(const VDesc& d);  // d = 2, 1 <= degree <= 4, chi <= 8
TcRec tc_record(const VDesc& d, const std::vector<long long>& msg_off);
void launch_build_zimg(const int* slot_vertex, int nslot, const VDesc* vd, const double* fac, __nv_bfloat16* zimg,
                       cudaStream_t s);
// Failure-detection test: extra bytes each tensor-core image copy's barrier expects.
void tc_set_test_extra_tx(unsigned int bytes);
void launch_tc_vertices(const TcRec* recs, int nwork, const __nv_bfloat16* zimg,
                        const float* msg_in, float* msg_out, double* diffs, const int* converged, int normalize,
                        int want_diff, int* err, cudaStream_t s);

// Adjoint kernels (adjoint.cu), FP64.
// Adjoint launchers: T = double or zdouble (complex cotangents are
// dL/dRe + i dL/dIm of a real loss).
size_t vertex_vjp_smem(int ncap, size_t elt = sizeof(double));
template <typename T>
void launch_site_op(int nv, const VDesc* vd, const T* fac, const T* op, T* out, cudaStream_t s);
template <typename T>
void launch_norm_vjp(int ndir, const int* dchi, const long long* msg_off, const T* f, const T* nbar, T* fbar,
                     cudaStream_t s);
template <typename T>
void launch_vertex_vjp(const int* work, int nwork, const VDesc* vd, const T* ket, const T* bra, const T* msgs,
                       const T* cot, const long long* msg_off, const T* op, T* mbar, T* abar, int ncap,
                       cudaStream_t s);
template <typename T>
void launch_edge_dot(int ne, const int* dchi, const long long* msg_off, const T* F, T* out, cudaStream_t s);
template <typename T>
void launch_energy_cot(int ndir, const int* dchi, const long long* msg_off, const T* F, const T* scale, T* C,
                       cudaStream_t s);
template <typename T>
void launch_energy_terms(int ne, int nterms, const double* coef, const T* t, double* Ee, T* scale, cudaStream_t s);
void launch_net_sum(int nnet, const int* net_e_ptr, const int* net_e, const double* Ee, double* out, cudaStream_t s);
void launch_phase_project(int ndir, const int* dchi, const long long* msg_off, const zdouble* m, zdouble* lam,
                          cudaStream_t s);
void launch_edge_phase(int ndir, const int* dchi, const long long* msg_off, const zdouble* m, const zdouble* f,
                       zdouble* rho, cudaStream_t s);
void launch_edge_rotate(int ndir, const int* dchi, const long long* msg_off, const zdouble* rho, const zdouble* in,
                        zdouble* out, cudaStream_t s);
template <typename T>
void launch_vertex_term_cot(int nv, const VDesc* vd, const long long* msg_off, const T* msgs, const T* F, const T* FO,
                            int mode, T* ci, T* co, T* g, double* val, cudaStream_t s);
template <typename T>
void launch_edge_term_cot(int ne, const int* dchi, const long long* msg_off, const T* msgs, T* g, double* val,
                          cudaStream_t s);
void launch_axpy_resid(long long n, const double* a, const double* b, const double* old, double* y, double* acc,
                       cudaStream_t s);

}  // namespace gbtn
