// Allocation-free FP64 BP sweep: gbtn_bp_sweep_static.
//
// Some callers of this library cannot call cudaMalloc at the point where they
// need a message update: code that runs while a CUDA stream is being
// captured into a graph by a host framework, or a host application that
// hands the library a fixed device memory budget and forbids allocation
// inside its solver loop.  They already own device buffers for the network
// and the messages, so this entry point takes only those and allocates
// nothing: its scratch memory (tensor offsets, message offsets, per-edge
// message diffs and a status word) lives in the file-scope array
// g_sweep_scratch below, of fixed size kScratchBytes (about 1.2 MiB).  Every
// GPU that loads the library holds that array until the process exits.
//
// The first call on a device looks up the array's device address with
// cudaGetSymbolAddress and raises the kernel's shared-memory limit; make that
// first call before any stream capture starts.  All calls share the array
// and it keeps the previous call's contents, so two calls whose work overlaps
// on the GPU (different streams, or different host threads) race with each
// other; serialise them.
#include <math.h>

#include <mutex>

#include "gbtn_internal.h"

namespace {

constexpr int kStaticMaxVertices = GBTN_STATIC_MAX_VERTICES;
constexpr int kStaticMaxDirected = GBTN_STATIC_MAX_DIRECTED_EDGES;
constexpr int kStaticMaxN = 8192;  // elements of one vertex tensor (3 buffers in shared memory)
constexpr int kThreads = 256;

// Scratch layout (bytes): vertex tensor offsets, message offsets, diffs, status.
constexpr size_t kVoffBytes = sizeof(long long) * (kStaticMaxVertices + 1);
constexpr size_t kMoffBytes = sizeof(long long) * (kStaticMaxDirected + 1);
constexpr size_t kDiffBytes = sizeof(double) * kStaticMaxDirected;
constexpr size_t kVoffAt = 0;
constexpr size_t kMoffAt = (kVoffAt + kVoffBytes + 255) / 256 * 256;
constexpr size_t kDiffAt = (kMoffAt + kMoffBytes + 255) / 256 * 256;
constexpr size_t kStatusAt = (kDiffAt + kDiffBytes + 255) / 256 * 256;
constexpr size_t kScratchBytes = kStatusAt + 256;

static __device__ __align__(256) unsigned char g_sweep_scratch[kScratchBytes];

struct Scratch {
  long long* voff;
  long long* moff;
  double* diff;
  int* status;
};

__device__ __forceinline__ Scratch view(unsigned char* base) {
  Scratch s;
  s.voff = reinterpret_cast<long long*>(base + kVoffAt);
  s.moff = reinterpret_cast<long long*>(base + kMoffAt);
  s.diff = reinterpret_cast<double*>(base + kDiffAt);
  s.status = reinterpret_cast<int*>(base + kStatusAt);
  return s;
}

__device__ __forceinline__ double wsum(double x) {
  for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Block-wide exclusive prefix sum of per-item sizes computed by size_of(i),
// items 0..n-1, written to out[0..n] (out[n] = total).  One block.
template <typename F>
__device__ void block_scan(int n, long long* out, F size_of) {
  __shared__ long long part[kThreads];
  const int per = (n + kThreads - 1) / kThreads;
  const int b = threadIdx.x * per, e = min(n, b + per);
  long long t = 0;
  for (int i = b; i < e; ++i) t += size_of(i);
  part[threadIdx.x] = t;
  __syncthreads();
  if (threadIdx.x == 0) {
    long long run = 0;
    for (int i = 0; i < kThreads; ++i) {
      const long long x = part[i];
      part[i] = run;
      run += x;
    }
    out[n] = run;
  }
  __syncthreads();
  long long run = part[threadIdx.x];
  for (int i = b; i < e; ++i) {
    out[i] = run;
    run += size_of(i);
  }
  __syncthreads();
}

// Structural checks of one vertex of a caller's device descriptor, made on the
// device before any array is indexed with a value read from the descriptor:
// leg_ptr non-decreasing with at most kMaxDeg legs, every leg edge in
// 0..ne-1 with v as one of its endpoints, bond and site dimensions >= 1.
// leg_edge is read only inside [leg_ptr[v], leg_ptr[v+1]), which the caller
// sizes (its length is leg_ptr[nv]).
__device__ __forceinline__ bool vertex_valid(const gbtn_graph_desc& g, int v) {
  const int b = g.leg_ptr[v], e_ = g.leg_ptr[v + 1];
  if (b < 0 || e_ < b || e_ - b > gbtn::kMaxDeg || g.site_dim[v] < 1) return false;
  for (int q = b; q < e_; ++q) {
    const int e = g.leg_edge[q];
    if (e < 0 || e >= g.ne) return false;
    if (g.edge_dim[e] < 1) return false;
    if (g.edge_u[e] != v && g.edge_v[e] != v) return false;
  }
  return true;
}

// Offsets of every vertex tensor and every message; status 0, or 1 when the
// descriptor fails a structural check (the offending sizes count as 0).
__global__ void __launch_bounds__(kThreads) static_prep_kernel(gbtn_graph_desc g, unsigned char* base) {
  Scratch S = view(base);
  __shared__ int s_bad;
  if (threadIdx.x == 0) s_bad = g.leg_ptr[0] != 0;
  __syncthreads();
  block_scan(g.nv, S.voff, [&](int v) -> long long {
    if (!vertex_valid(g, v)) {
      s_bad = 1;
      return 0;
    }
    long long n = g.site_dim[v];
    for (int q = g.leg_ptr[v]; q < g.leg_ptr[v + 1]; ++q) n *= g.edge_dim[g.leg_edge[q]];
    return n;
  });
  block_scan(2 * g.ne, S.moff, [&](int de) -> long long {
    const long long c = g.edge_dim[de >> 1];
    if (c < 1) {
      s_bad = 1;
      return 0;
    }
    return c * c;
  });
  if (threadIdx.x == 0) *S.status = s_bad;
}

__device__ __forceinline__ void absorb_leg(const double* in, double* out, int n, int st, int chi, const double* M) {
  const int nfib = n / chi;
  for (int f = threadIdx.x; f < nfib; f += kThreads) {
    const int lo = f % st;
    const int base = lo + (f - lo) * chi;
    double x[gbtn::kMaxChi];
    for (int a = 0; a < chi; ++a) x[a] = in[base + a * st];
    for (int b = 0; b < chi; ++b) {
      double y = 0.0;
      for (int a = 0; a < chi; ++a) y = fma(M[b + chi * a], x[a], y);
      out[base + b * st] = y;
    }
  }
}

// res[b + chi*a] = sum over fibers of bra[.., b, ..] * t[.., a, ..]; one value
// per thread slot, reduced through shared memory.
__device__ void close_leg(const double* t, const double* bra, int n, int st, int chi, double* red, double* res) {
  const int P = chi * chi;
  const int nfib = n / chi;
  // thread j accumulates output o = j % P over fibers f = j / P, j / P + G, ...
  const int G = kThreads / P;
  const int o = threadIdx.x % P, g0 = threadIdx.x / P;
  double acc = 0.0;
  if (g0 < G) {
    const int b = o % chi, a = o / chi;
    for (int f = g0; f < nfib; f += G) {
      const int lo = f % st;
      const int base = lo + (f - lo) * chi;
      acc = fma(bra[base + b * st], t[base + a * st], acc);
    }
  }
  red[threadIdx.x] = acc;
  __syncthreads();
  if (threadIdx.x < P) {
    double s = 0.0;
    for (int q = 0; q < G; ++q) s += red[threadIdx.x + q * P];
    res[threadIdx.x] = s;
  }
  __syncthreads();
}

// One block per vertex: every outgoing message from msg_in into msg_out,
// normalised in FP64, with its message diff in the scratch array.
__global__ void __launch_bounds__(kThreads)
    static_sweep_kernel(gbtn_graph_desc g, const double* __restrict__ fac, const double* __restrict__ msg_in,
                        double* __restrict__ msg_out, unsigned char* base) {
  extern __shared__ __align__(16) double sm[];
  __shared__ int s_chi[gbtn::kMaxDeg], s_st[gbtn::kMaxDeg], s_in[gbtn::kMaxDeg], s_out[gbtn::kMaxDeg];
  __shared__ int s_k, s_n, s_ok;
  __shared__ long long s_aoff;
  Scratch S = view(base);
  const int v = blockIdx.x;
  if (threadIdx.x == 0) {
    int ok = vertex_valid(g, v);
    const int k = ok ? g.leg_ptr[v + 1] - g.leg_ptr[v] : 0;
    const int d = g.site_dim[v];
    const long long n = S.voff[v + 1] - S.voff[v];
    ok = ok && d <= gbtn::kMaxSite && n <= kStaticMaxN;
    long long st = d;
    for (int p = 0; ok && p < k; ++p) {
      const int e = g.leg_edge[g.leg_ptr[v] + p];
      const int c = g.edge_dim[e];
      ok = ok && c <= gbtn::kMaxChi;
      s_chi[p] = c;
      s_st[p] = (int)st;
      st *= c;
      s_out[p] = g.edge_u[e] == v ? 2 * e : 2 * e + 1;
      s_in[p] = s_out[p] ^ 1;
    }
    ok = ok && st == n;  // the offsets agree with this vertex's own shape
    s_k = k;
    s_n = (int)n;
    s_aoff = S.voff[v];
    s_ok = ok;
    if (!ok) atomicExch(S.status, 1);
  }
  __syncthreads();
  if (!s_ok) return;
  const int k = s_k, n = s_n;
  double* A = sm;
  double* B1 = sm + kStaticMaxN;
  double* B2 = sm + 2 * kStaticMaxN;
  double* M = sm + 3 * kStaticMaxN;      // kMaxDeg x 64
  double* red = M + gbtn::kMaxDeg * 64;  // kThreads
  double* res = red + kThreads;          // 64
  for (int i = threadIdx.x; i < n; i += kThreads) A[i] = fac[s_aoff + i];
  for (int p = 0; p < k; ++p) {
    const int c2 = s_chi[p] * s_chi[p];
    for (int i = threadIdx.x; i < c2; i += kThreads) M[p * 64 + i] = msg_in[S.moff[s_in[p]] + i];
  }
  __syncthreads();
  for (int w = 0; w < k; ++w) {
    const double* cur = A;
    double* bufs[2] = {B1, B2};
    int which = 0;
    for (int j = 0; j < k; ++j) {
      if (j == w) continue;
      absorb_leg(cur, bufs[which], n, s_st[j], s_chi[j], M + j * 64);
      __syncthreads();
      cur = bufs[which];
      which ^= 1;
    }
    close_leg(cur, A, n, s_st[w], s_chi[w], red, res);
    if (threadIdx.x < 32) {
      const int lane = threadIdx.x;
      const int P = s_chi[w] * s_chi[w];
      const long long off = S.moff[s_out[w]];
      const double x0 = lane < P ? res[lane] : 0.0, x1 = lane + 32 < P ? res[lane + 32] : 0.0;
      const double nrm2 = wsum(x0 * x0 + x1 * x1);
      const double sc = nrm2 > 0.0 ? 1.0 / sqrt(nrm2) : 1.0;
      const double y0 = x0 * sc, y1 = x1 * sc;
      const double o0 = lane < P ? msg_in[off + lane] : 0.0, o1 = lane + 32 < P ? msg_in[off + lane + 32] : 0.0;
      if (lane < P) msg_out[off + lane] = y0;
      if (lane + 32 < P) msg_out[off + lane + 32] = y1;
      const double dot = wsum(y0 * o0 + y1 * o1), na = wsum(y0 * y0 + y1 * y1), nb = wsum(o0 * o0 + o1 * o1);
      if (lane == 0) S.diff[s_out[w]] = 1.0 - (dot * dot) / (na * nb);
    }
    __syncthreads();
  }
}

// mean over every directed edge of the message diffs, or NaN after a
// rejected vertex.
__global__ void __launch_bounds__(kThreads) static_mean_kernel(int ndir, unsigned char* base, double* mean_out) {
  Scratch S = view(base);
  __shared__ double part[kThreads / 32];
  double s = 0.0;
  for (int i = threadIdx.x; i < ndir; i += kThreads) s += S.diff[i];
  s = wsum(s);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < kThreads / 32; ++w) t += part[w];
    *mean_out = *S.status ? NAN : (ndir ? t / ndir : 0.0);
  }
}

constexpr size_t kSweepSmem = sizeof(double) * (3 * (size_t)kStaticMaxN + gbtn::kMaxDeg * 64 + kThreads + 64);

// Per-device set-up: the scratch array's device address and the sweep
// kernel's shared-memory limit.  A set-up that fails (for example a first
// call made during a stream capture) is retried by the next call.
struct DeviceSetup {
  std::mutex mu;
  unsigned char* ptr = nullptr;
  bool done = false;
};
DeviceSetup g_setup[64];

cudaError_t setup_device(DeviceSetup& ds) {
  std::lock_guard<std::mutex> lock(ds.mu);
  if (ds.done) return cudaSuccess;
  unsigned char* p = nullptr;
  cudaError_t err = cudaGetSymbolAddress(reinterpret_cast<void**>(&p), g_sweep_scratch);
  if (err == cudaSuccess)
    err = cudaFuncSetAttribute(static_sweep_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kSweepSmem);
  if (err != cudaSuccess || !p) {
    cudaGetLastError();  // a failed set-up leaves no sticky error for the caller's next launch
    return err != cudaSuccess ? err : cudaErrorInvalidSymbol;
  }
  ds.ptr = p;
  ds.done = true;
  return cudaSuccess;
}

}  // namespace

extern "C" {

int gbtn_bp_sweep_static(int device, const gbtn_graph_desc* g, const double* fac, const double* msg_in,
                         double* msg_out, double* mean_diff, void* stream) {
  if (!g || !fac || !msg_in || !msg_out || !mean_diff) {
    return GBTN_ERR_INVALID;
  }
  if (device < 0 || device >= 64) {
    return GBTN_ERR_INVALID;
  }
  if (g->nv < 1 || g->ne < 0 || g->nv > kStaticMaxVertices || 2LL * g->ne > kStaticMaxDirected ||
      g->complex_values || g->separate_bra) {
    return GBTN_ERR_UNSUPPORTED;
  }
  if (!g->site_dim || !g->leg_ptr || (g->ne > 0 && (!g->edge_dim || !g->edge_u || !g->edge_v || !g->leg_edge))) {
    return GBTN_ERR_INVALID;
  }
  int prev = 0;
  if (cudaGetDevice(&prev) != cudaSuccess) {
    return GBTN_ERR_CUDA;
  }
  if (prev != device && cudaSetDevice(device) != cudaSuccess) {
    return GBTN_ERR_CUDA;
  }
  DeviceSetup& ds = g_setup[device];
  int rc = GBTN_OK;
  if (setup_device(ds) != cudaSuccess) {
    rc = GBTN_ERR_CUDA;
  } else {
    cudaStream_t s = reinterpret_cast<cudaStream_t>(stream);
    static_prep_kernel<<<1, kThreads, 0, s>>>(*g, ds.ptr);
    static_sweep_kernel<<<g->nv, kThreads, kSweepSmem, s>>>(*g, fac, msg_in, msg_out, ds.ptr);
    static_mean_kernel<<<1, kThreads, 0, s>>>(2 * g->ne, ds.ptr, mean_diff);
    const cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        rc = GBTN_ERR_CUDA;
    }
  }
  if (prev != device) cudaSetDevice(prev);
  return rc;
}

}  // extern "C"
