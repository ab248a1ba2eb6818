// Hand-written adjoints of the BP hot path (FP64).
//
// The reference has no automatic differentiation; these kernels are the
// reverse-mode rules of the forward kernels:
//
//  * vertex VJP.  For one vertex with ket tensor K (A_v, or O.A_v with a site
//    operator O applied), bra A_v, incoming messages m_q and cotangents C_w of
//    its unnormalised outgoing messages F_w = CLOSE_w(K absorbed with m_q, q != w):
//      L = sum_w <C_w, F_w> = sum_w sum K[s,a] A[s,b] prod_q M^(w)_q[b_q, a_q],
//      M^(w)_q = m_q (q != w), C_w (q = w);
//      dL/dm_p  = sum_{w != p} CLOSE_p(K absorbed with M^(w)_q, q != p)
//      dL/dK    = sum_w A absorbed with every (M^(w)_q)^T,
//      dL/dA    = O^T dL/dK + sum_w K absorbed with every M^(w)_q.
//  * normalisation VJP: n = f/|f|  =>  f_bar = (n_bar - <n, n_bar> n) / |f|
//    (updated_message's division by the norm,
//    src/caches/abstractbeliefpropagationcache.jl:234-237).
//  * two-site energy terms: with F^O the message computed with O applied to the
//    ket, tr(rho_e (O (x) O)) = <F^O_{u->v}, F^O_{v->u}> (Frobenius), so
//    E = sum_e sum_t c_t <F^{O_t}_{u->v}, F^{O_t}_{v->u}> / <F^I_{u->v}, F^I_{v->u}>
//    and its cotangents on F^{O_t} are products of the opposite messages.
// The host side (api.cu) chains them into the implicit adjoint at the BP fixed
// point (iterating lambda <- dE/dm + (dF/dm)^T lambda) and into backpropagation
// through unrolled, checkpointed Jacobi sweeps.
#include "bp_device.cuh"

namespace gbtn {
namespace {

// out[v] = O . A_v on the site index (O[s', s], d x d, column-major).
template <typename T>
__global__ void site_op_kernel(int nv, const VDesc* __restrict__ vd, const T* __restrict__ fac,
                               const T* __restrict__ op, T* __restrict__ out) {
  const int v = blockIdx.x;
  if (v >= nv) return;
  const VDesc d = vd[v];
  const T* a = fac + d.a_off;
  T* o = out + d.a_off;
  for (int i = threadIdx.x; i < d.n; i += blockDim.x) {
    const int s = i % d.d, r = i - s;
    T acc = T(0);
    for (int t = 0; t < d.d; ++t) acc = mac(op[s + d.d * t], a[r + t], acc);
    o[i] = acc;
  }
}

__device__ __forceinline__ double re_of(double x) { return x; }
__device__ __forceinline__ double re_of(zdouble x) { return x.re; }
__device__ __forceinline__ double abs2(double x) { return x * x; }
__device__ __forceinline__ double abs2(zdouble x) { return x.re * x.re + x.im * x.im; }
__device__ __forceinline__ zdouble operator*(zdouble a, zdouble b) {
  return zdouble(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ zdouble operator*(double a, zdouble b) { return zdouble(a * b.re, a * b.im); }
__device__ __forceinline__ zdouble operator-(zdouble a, zdouble b) { return zdouble(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ zdouble zwarp_sum(zdouble x) { return zdouble(warp_sum(x.re), warp_sum(x.im)); }
__device__ __forceinline__ double zwarp_sum(double x) { return warp_sum(x); }
__device__ __forceinline__ double inv_of(double x) { return 1.0 / x; }
__device__ __forceinline__ zdouble inv_of(zdouble x) {
  const double r = 1.0 / (x.re * x.re + x.im * x.im);
  return zdouble(x.re * r, -x.im * r);
}
__device__ __forceinline__ double log_abs(double x) { return log(fabs(x)); }
__device__ __forceinline__ double log_abs(zdouble x) { return 0.5 * log(x.re * x.re + x.im * x.im); }

// Normalisation VJP per directed edge (one warp each).  Complex entries (the
// cotangent of a real loss being dL/dRe + i dL/dIm): with n = f / |f|,
// f_bar = (n_bar - n Re<n, n_bar>) / |f|, <x, y> = sum conj(x) y.
template <typename T>
__global__ void norm_vjp_kernel(int ndir, const int* __restrict__ dchi, const long long* __restrict__ msg_off,
                                const T* __restrict__ f, const T* __restrict__ nbar, T* __restrict__ fbar) {
  const int de = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (de >= ndir) return;
  const int c2 = dchi[de] * dchi[de];
  const long long off = msg_off[de];
  const T zero = T(0);
  const T f0 = lane < c2 ? f[off + lane] : zero, f1 = lane + 32 < c2 ? f[off + lane + 32] : zero;
  const T g0 = lane < c2 ? nbar[off + lane] : zero, g1 = lane + 32 < c2 ? nbar[off + lane + 32] : zero;
  const double nrm = sqrt(warp_sum(abs2(f0) + abs2(f1)));
  T r0 = zero, r1 = zero;
  if (nrm > 0.0) {
    const double inv = 1.0 / nrm;
    const double dot = warp_sum(re_of(conj_of(f0) * g0) + re_of(conj_of(f1) * g1)) * inv;  // Re<n, n_bar>
    r0 = inv * (g0 - (dot * inv) * f0);
    r1 = inv * (g1 - (dot * inv) * f1);
  }
  if (lane < c2) fbar[off + lane] = r0;
  if (lane + 32 < c2) fbar[off + lane + 32] = r1;
}

// One CTA per vertex (256 threads); see the file comment.  mbar / abar may be
// NULL to skip that part.  Results are accumulated (+=): mbar by incoming
// directed edge (each one belongs to exactly one vertex), abar by tensor entry.
//
// Complex tensors (T = zdouble; the forward message is
// F_w = sum conj(A[s,b]) K[s,a] prod m, and a cotangent is dL/dRe + i dL/dIm
// of a real loss): with the outgoing cotangents conjugated on load (Cc = conj C),
//   dL/dm_p = conj(CLOSE_p(K absorbed with m_q and Cc_w, bra A)),
//   dL/dK   = conj(conj(A) absorbed with every m_q^T and Cc_w^T),
//   dL/dA   = O^H dL/dK + K absorbed with every m_q and Cc_w;
// every conj is the identity for real tensors, which gives the real rules.
constexpr int kVjpTeam = 256;

template <typename T>
__global__ void __launch_bounds__(kVjpTeam)
    vertex_vjp_kernel(const int* __restrict__ work, int nwork, const VDesc* __restrict__ vd,
                      const T* __restrict__ ket, const T* __restrict__ bra, const T* __restrict__ msgs,
                      const T* __restrict__ cot, const long long* __restrict__ msg_off, const T* __restrict__ op,
                      T* mbar, T* abar, int ncap) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  constexpr int TEAM = kVjpTeam;
  const int tid = threadIdx.x;
  VDesc* D = reinterpret_cast<VDesc*>(smem_raw);
  T* base = reinterpret_cast<T*>(smem_raw + align_up(sizeof(VDesc), 16));
  T* K = base;
  T* B = K + ncap;
  T* W[2] = {B + ncap, B + 2 * (size_t)ncap};
  T* GK = B + 3 * (size_t)ncap;
  T* GB = B + 4 * (size_t)ncap;
  T* MS = B + 5 * (size_t)ncap;  // incoming messages, kMaxDeg x 64
  T* CT = MS + kMaxDeg * 64;     // conjugated cotangents of outgoing messages, kMaxDeg x 64
  T* MT = CT + kMaxDeg * 64;     // one transposed message
  T* MB = MT + 64;               // accumulated incoming-message cotangents, kMaxDeg x 64
  T* red = MB + kMaxDeg * 64;    // (TEAM/32) x kRedStride
  T* res = red + (TEAM / 32) * kRedStride;
  const T zero = T(0);
  for (int w_ = blockIdx.x; w_ < nwork; w_ += gridDim.x) {
    const int v = work[w_];
    load_desc<TEAM>(D, vd + v, tid);
    __syncthreads();
    const VDesc& d = *D;
    const int n = d.n, k = d.k;
    for (int i = tid; i < n; i += TEAM) {
      K[i] = ket[d.a_off + i];
      B[i] = bra[d.a_off + i];
      GK[i] = zero;
      GB[i] = zero;
    }
    for (int p = 0; p < k; ++p) {
      const int c2 = d.chi[p] * d.chi[p];
      for (int i = tid; i < c2; i += TEAM) {
        MS[p * 64 + i] = msgs[msg_off[d.in_de[p]] + i];
        CT[p * 64 + i] = conj_of(cot[msg_off[d.out_de[p]] + i]);
        MB[p * 64 + i] = zero;
      }
    }
    __syncthreads();
    if (mbar) {
      for (int w = 0; w < k; ++w)
        for (int p = 0; p < k; ++p) {
          if (p == w) continue;
          const T* cur = K;
          int nx = 0;
          for (int q = 0; q < k; ++q) {
            if (q == p) continue;
            absorb_any<T>(d.chi[q], cur, W[nx], n, d.st[q], q == w ? CT + w * 64 : MS + q * 64, tid, TEAM);
            __syncthreads();
            cur = W[nx];
            nx ^= 1;
          }
          close_any<T, TEAM>(d.chi[p], cur, B, n, d.st[p], 1, 0, 0, red, res, tid);
          for (int i = tid; i < d.chi[p] * d.chi[p]; i += TEAM) MB[p * 64 + i] += conj_of(res[i]);
          __syncthreads();
        }
      for (int p = 0; p < k; ++p) {
        const int c2 = d.chi[p] * d.chi[p];
        const long long off = msg_off[d.in_de[p]];
        for (int i = tid; i < c2; i += TEAM) mbar[off + i] += MB[p * 64 + i];
      }
    }
    if (abar) {
      if constexpr (!std::is_same<T, double>::value) {
        // the ket-side rule reads conj(A); the incoming-message part above was
        // the only other reader of B
        for (int i = tid; i < n; i += TEAM) B[i] = conj_of(B[i]);
        __syncthreads();
      }
      for (int w = 0; w < k; ++w) {
        // dL/dK: conj(A) absorbed with every transposed message, conjugated at the end
        const T* cur = B;
        int nx = 0;
        for (int q = 0; q < k; ++q) {
          const int c = d.chi[q];
          const T* M = q == w ? CT + w * 64 : MS + q * 64;
          for (int i = tid; i < c * c; i += TEAM) MT[(i / c) + c * (i % c)] = M[i];
          __syncthreads();
          absorb_any<T>(c, cur, W[nx], n, d.st[q], MT, tid, TEAM);
          __syncthreads();
          cur = W[nx];
          nx ^= 1;
        }
        for (int i = tid; i < n; i += TEAM) GK[i] += conj_of(cur[i]);
        __syncthreads();
        // dL/dA (bra side): the ket absorbed with every message
        cur = K;
        for (int q = 0; q < k; ++q) {
          absorb_any<T>(d.chi[q], cur, W[nx], n, d.st[q], q == w ? CT + w * 64 : MS + q * 64, tid, TEAM);
          __syncthreads();
          cur = W[nx];
          nx ^= 1;
        }
        for (int i = tid; i < n; i += TEAM) GB[i] += cur[i];
        __syncthreads();
      }
      // abar += O^H . GK + GB
      for (int i = tid; i < n; i += TEAM) {
        const int s = i % d.d, r = i - s;
        T acc = GB[i];
        for (int t = 0; t < d.d; ++t) {
          if (op)
            acc = mac(conj_of(op[t + d.d * s]), GK[r + t], acc);
          else if (t == s)
            acc += GK[r + t];
        }
        abar[d.a_off + i] += acc;
      }
    }
    __syncthreads();
  }
}

// Complex networks: remove from a message cotangent lam its component along the
// message's own phase direction i m (real inner product Im<m, lam>), one warp
// per directed edge.  Every loss built from region scalars is invariant under
// a phase per message, and the BP Jacobian maps those phase directions into
// themselves with gain ~3 per sweep (the phase of m_{u->v} reaches every
// m_{v->w}), so the adjoint solution has no such component while rounding in
// the adjoint iteration would feed one that grows threefold per iteration.
__global__ void phase_project_kernel(int ndir, const int* __restrict__ dchi, const long long* __restrict__ msg_off,
                                     const zdouble* __restrict__ m, zdouble* lam) {
  const int de = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (de >= ndir) return;
  const int c2 = dchi[de] * dchi[de];
  const long long off = msg_off[de];
  double im = 0.0, n2 = 0.0;
  for (int i = lane; i < c2; i += 32) {
    const zdouble a = m[off + i], b = lam[off + i];
    im += a.re * b.im - a.im * b.re;
    n2 += a.re * a.re + a.im * a.im;
  }
  im = warp_sum(im);
  n2 = warp_sum(n2);
  if (n2 <= 0.0) return;
  const double t = im / n2;
  for (int i = lane; i < c2; i += 32) {
    const zdouble a = m[off + i];
    lam[off + i] = zdouble(lam[off + i].re + t * a.im, lam[off + i].im - t * a.re);
  }
}

// Complex networks: the phase by which one sweep moves each message.  BP on a
// loopy complex network does not settle the phases of its messages (they
// drift), so one sweep from the converged messages m returns n = R m with R a
// unit complex factor per message, rho_e = <m_e, f_e> / |<m_e, f_e>|
// (f the unnormalised update).  The adjoint linearises f^ = R^-1 f, which has
// m as its exact fixed point; every loss here is invariant under message
// phases, so its value and gradient are those of the quotient, and
// (df^/dm)^H = (df/dm)^H R: each message cotangent is multiplied by rho_e
// before the VJP of the update.  One warp per directed edge.
__global__ void edge_phase_kernel(int ndir, const int* __restrict__ dchi, const long long* __restrict__ msg_off,
                                  const zdouble* __restrict__ m, const zdouble* __restrict__ f, zdouble* rho) {
  const int de = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (de >= ndir) return;
  const int c2 = dchi[de] * dchi[de];
  const long long off = msg_off[de];
  double re = 0.0, im = 0.0;
  for (int i = lane; i < c2; i += 32) {
    const zdouble a = m[off + i], b = f[off + i];
    re += a.re * b.re + a.im * b.im;
    im += a.re * b.im - a.im * b.re;
  }
  re = warp_sum(re);
  im = warp_sum(im);
  if (lane == 0) {
    const double r = sqrt(re * re + im * im);
    rho[de] = r > 0.0 ? zdouble(re / r, im / r) : zdouble(1.0, 0.0);
  }
}

// out_e = rho_e * in_e per directed edge (one warp each).
__global__ void edge_rotate_kernel(int ndir, const int* __restrict__ dchi, const long long* __restrict__ msg_off,
                                   const zdouble* __restrict__ rho, const zdouble* __restrict__ in, zdouble* out) {
  const int de = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (de >= ndir) return;
  const int c2 = dchi[de] * dchi[de];
  const long long off = msg_off[de];
  const zdouble r = rho[de];
  for (int i = lane; i < c2; i += 32) out[off + i] = r * in[off + i];
}

// Per edge: t[e] = sum F[2e] F[2e+1] (bilinear; one warp per edge).
template <typename T>
__global__ void edge_dot_kernel(int ne, const int* __restrict__ dchi, const long long* __restrict__ msg_off,
                                const T* __restrict__ F, T* __restrict__ out) {
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= ne) return;
  const int c2 = dchi[2 * e] * dchi[2 * e];
  T s = T(0);
  for (int i = lane; i < c2; i += 32) s = mac(F[msg_off[2 * e] + i], F[msg_off[2 * e + 1] + i], s);
  s = zwarp_sum(s);
  if (lane == 0) out[e] = s;
}

// Cotangents of the energy on the term messages: for directed edge de of edge e,
// C[de] = conj(scale[e] * F[de ^ 1]) (scale = c_t / t_I for an operator term,
// -E_e / t_I for the identity term; the conjugate is the identity for real tensors).
template <typename T>
__global__ void energy_cot_kernel(int ndir, const int* __restrict__ dchi, const long long* __restrict__ msg_off,
                                  const T* __restrict__ F, const T* __restrict__ scale, T* __restrict__ C) {
  const int de = blockIdx.x;
  if (de >= ndir) return;
  const int c2 = dchi[de] * dchi[de];
  const T sc = scale[de >> 1];
  for (int i = threadIdx.x; i < c2; i += blockDim.x) C[msg_off[de] + i] = conj_of(sc * F[msg_off[de ^ 1] + i]);
}

}  // namespace

namespace {

// Per edge: E_e = sum_t c_t t[t][e] / t[I][e] and the cotangent scales
// scale[t][e] = c_t / t[I][e], scale[I][e] = -E_e / t[I][e] (term 0 = identity);
// Ee receives Re E_e (the energy of a complex network is its real part).
template <typename T>
__global__ void energy_terms_kernel(int ne, int nterms, const double* __restrict__ coef, const T* __restrict__ t,
                                    double* __restrict__ Ee, T* __restrict__ scale) {
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e >= ne) return;
  const T itI = inv_of(t[e]);
  T E = T(0);
  for (int k = 1; k <= nterms; ++k) {
    E = mac(T(coef[k - 1]) * itI, t[(size_t)k * ne + e], E);
    scale[(size_t)k * ne + e] = T(coef[k - 1]) * itI;
  }
  Ee[e] = re_of(E);
  scale[e] = T(0) - E * itI;
}

// Per network: sum of its edges' energies.
__global__ void net_sum_kernel(const int* __restrict__ net_e_ptr, const int* __restrict__ net_e,
                               const double* __restrict__ Ee, double* __restrict__ out) {
  const int net = blockIdx.x;
  double s = 0.0;
  for (int i = net_e_ptr[net] + threadIdx.x; i < net_e_ptr[net + 1]; i += blockDim.x) s += Ee[net_e[i]];
  __shared__ double red[32];
  s = warp_sum(s);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
    out[net] = t;
  }
}

// y = a + b (elementwise) and the squared norms of y and y - old.
__global__ void axpy_resid_kernel(long long n, const double* __restrict__ a, const double* __restrict__ b,
                                  const double* __restrict__ old, double* __restrict__ y, double* __restrict__ acc) {
  double s_new = 0.0, s_diff = 0.0;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
    const double v = a[i] + b[i];
    const double dlt = v - old[i];
    y[i] = v;
    s_new += v * v;
    s_diff += dlt * dlt;
  }
  s_new = warp_sum(s_new);
  s_diff = warp_sum(s_diff);
  if ((threadIdx.x & 31) == 0) {
    atomicAdd(&acc[0], s_new);
    atomicAdd(&acc[1], s_diff);
  }
}

}  // namespace

size_t vertex_vjp_smem(int ncap, size_t elt) {
  return align_up(sizeof(VDesc), 16) +
         elt * (6 * (size_t)ncap + 3 * kMaxDeg * 64 + 64 + (kVjpTeam / 32) * kRedStride + 64);
}

template <typename T>
void launch_site_op(int nv, const VDesc* vd, const T* fac, const T* op, T* out, cudaStream_t s) {
  site_op_kernel<T><<<nv, 256, 0, s>>>(nv, vd, fac, op, out);
  GBTN_CUDA(cudaGetLastError());
}

// Vertex terms of the log-norm and of one-site expectation values, as
// contractions of an unnormalised outgoing message with the incoming one on
// the same leg (leg 0 of every vertex): the full contraction of a partition is
// D_v = <F_{v->w}, m_{w->v}> = sum F m (bilinear; region_scalar,
// beliefpropagationcache.jl:107-113), and with O applied to the ket
// N_v = sum F^O m = tr(rho_v O).  One warp per vertex (degree >= 1).  The loss
// is real: log|D_v| = Re log D_v, and Re(N_v / D_v); a cotangent is the
// conjugate of the holomorphic derivative (dL/dRe + i dL/dIm), which for real
// tensors is the derivative itself.
//   mode 0 (log-norm, logscalar abstractbeliefpropagationcache.jl:397-408):
//     val[v] = log|D_v|; cotangent of F_{v->w}: conj(m_{w->v} / D_v) (into ci);
//     g[w->v] += conj(F_{v->w} / D_v).
//   mode 1 (expect, expect.jl:5-19): val[v] = Re(N_v / D_v); cotangents
//     co (of F^O_{v->w}) = conj(m / D_v) and ci (of F_{v->w}) = conj(-N_v / D_v^2 m);
//     g[w->v] += conj(F^O / D_v - N_v / D_v^2 F).

template <typename T>
__global__ void vertex_term_cot_kernel(int nv, const VDesc* __restrict__ vd, const long long* __restrict__ msg_off,
                                       const T* __restrict__ msgs, const T* __restrict__ F,
                                       const T* __restrict__ FO, int mode, T* ci, T* co, T* g, double* val) {
  const int v = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (v >= nv) return;
  const VDesc& d = vd[v];
  const int c2 = d.chi[0] * d.chi[0];
  const long long oo = msg_off[d.out_de[0]], oi = msg_off[d.in_de[0]];
  T dd = T(0), nn = T(0);
  for (int i = lane; i < c2; i += 32) {
    dd = mac(F[oo + i], msgs[oi + i], dd);
    if (mode == 1) nn = mac(FO[oo + i], msgs[oi + i], nn);
  }
  dd = zwarp_sum(dd);
  nn = zwarp_sum(nn);
  const T inv = inv_of(dd);
  if (mode == 0) {
    for (int i = lane; i < c2; i += 32) {
      ci[oo + i] = conj_of(msgs[oi + i] * inv);
      g[oi + i] += conj_of(F[oo + i] * inv);
    }
    if (lane == 0) val[v] = log_abs(dd);
  } else {
    const T r = nn * inv * inv;
    for (int i = lane; i < c2; i += 32) {
      co[oo + i] = conj_of(msgs[oi + i] * inv);
      ci[oo + i] = conj_of(T(0) - r * msgs[oi + i]);
      g[oi + i] += conj_of(FO[oo + i] * inv - r * F[oo + i]);
    }
    if (lane == 0) val[v] = re_of(nn * inv);
  }
}

// Edge terms of the log-norm: z_e = sum m_e m_ebar, val[e] = log|z_e|,
// g[e] -= conj(m_ebar / z_e) and g[ebar] -= conj(m_e / z_e).  One warp per edge.
template <typename T>
__global__ void edge_term_cot_kernel(int ne, const int* __restrict__ dchi, const long long* __restrict__ msg_off,
                                     const T* __restrict__ msgs, T* g, double* val) {
  const int e = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (e >= ne) return;
  const int c2 = dchi[2 * e] * dchi[2 * e];
  const long long o1 = msg_off[2 * e], o2 = msg_off[2 * e + 1];
  T z = T(0);
  for (int i = lane; i < c2; i += 32) z = mac(msgs[o1 + i], msgs[o2 + i], z);
  z = zwarp_sum(z);
  const T inv = inv_of(z);
  for (int i = lane; i < c2; i += 32) {
    const T a = msgs[o1 + i], b = msgs[o2 + i];
    g[o1 + i] = g[o1 + i] - conj_of(b * inv);
    g[o2 + i] = g[o2 + i] - conj_of(a * inv);
  }
  if (lane == 0) val[e] = log_abs(z);
}

template <typename T>
void launch_vertex_term_cot(int nv, const VDesc* vd, const long long* msg_off, const T* msgs, const T* F,
                            const T* FO, int mode, T* ci, T* co, T* g, double* val, cudaStream_t s) {
  if (nv == 0) return;
  vertex_term_cot_kernel<T><<<(nv + 7) / 8, 256, 0, s>>>(nv, vd, msg_off, msgs, F, FO, mode, ci, co, g, val);
  GBTN_CUDA(cudaGetLastError());
}

template <typename T>
void launch_edge_term_cot(int ne, const int* dchi, const long long* msg_off, const T* msgs, T* g, double* val,
                          cudaStream_t s) {
  if (ne == 0) return;
  edge_term_cot_kernel<T><<<(ne + 7) / 8, 256, 0, s>>>(ne, dchi, msg_off, msgs, g, val);
  GBTN_CUDA(cudaGetLastError());
}

template <typename T>
void launch_norm_vjp(int ndir, const int* dchi, const long long* msg_off, const T* f, const T* nbar, T* fbar,
                     cudaStream_t s) {
  if (ndir == 0) return;
  norm_vjp_kernel<T><<<(ndir + 7) / 8, 256, 0, s>>>(ndir, dchi, msg_off, f, nbar, fbar);
  GBTN_CUDA(cudaGetLastError());
}

template <typename T>
void launch_vertex_vjp(const int* work, int nwork, const VDesc* vd, const T* ket, const T* bra, const T* msgs,
                       const T* cot, const long long* msg_off, const T* op, T* mbar, T* abar, int ncap,
                       cudaStream_t s) {
  if (nwork == 0) return;
  const size_t sm = vertex_vjp_smem(ncap, sizeof(T));
  GBTN_CUDA(cudaFuncSetAttribute(vertex_vjp_kernel<T>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  vertex_vjp_kernel<T><<<nwork, kVjpTeam, sm, s>>>(work, nwork, vd, ket, bra, msgs, cot, msg_off, op, mbar, abar,
                                                   ncap);
  GBTN_CUDA(cudaGetLastError());
}

void launch_phase_project(int ndir, const int* dchi, const long long* msg_off, const zdouble* m, zdouble* lam,
                          cudaStream_t s) {
  if (ndir == 0) return;
  phase_project_kernel<<<(ndir + 7) / 8, 256, 0, s>>>(ndir, dchi, msg_off, m, lam);
  GBTN_CUDA(cudaGetLastError());
}

void launch_edge_phase(int ndir, const int* dchi, const long long* msg_off, const zdouble* m, const zdouble* f,
                       zdouble* rho, cudaStream_t s) {
  if (ndir == 0) return;
  edge_phase_kernel<<<(ndir + 7) / 8, 256, 0, s>>>(ndir, dchi, msg_off, m, f, rho);
  GBTN_CUDA(cudaGetLastError());
}

void launch_edge_rotate(int ndir, const int* dchi, const long long* msg_off, const zdouble* rho, const zdouble* in,
                        zdouble* out, cudaStream_t s) {
  if (ndir == 0) return;
  edge_rotate_kernel<<<(ndir + 7) / 8, 256, 0, s>>>(ndir, dchi, msg_off, rho, in, out);
  GBTN_CUDA(cudaGetLastError());
}

#define GBTN_ADJOINT_INSTANTIATE(T)                                                                                \
  template void launch_site_op<T>(int, const VDesc*, const T*, const T*, T*, cudaStream_t);                        \
  template void launch_vertex_term_cot<T>(int, const VDesc*, const long long*, const T*, const T*, const T*, int,  \
                                          T*, T*, T*, double*, cudaStream_t);                                      \
  template void launch_edge_term_cot<T>(int, const int*, const long long*, const T*, T*, double*, cudaStream_t);   \
  template void launch_norm_vjp<T>(int, const int*, const long long*, const T*, const T*, T*, cudaStream_t);       \
  template void launch_vertex_vjp<T>(const int*, int, const VDesc*, const T*, const T*, const T*, const T*,        \
                                     const long long*, const T*, T*, T*, int, cudaStream_t);
GBTN_ADJOINT_INSTANTIATE(double)
GBTN_ADJOINT_INSTANTIATE(zdouble)
#undef GBTN_ADJOINT_INSTANTIATE

template <typename T>
void launch_edge_dot(int ne, const int* dchi, const long long* msg_off, const T* F, T* out, cudaStream_t s) {
  if (ne == 0) return;
  edge_dot_kernel<T><<<(ne + 7) / 8, 256, 0, s>>>(ne, dchi, msg_off, F, out);
  GBTN_CUDA(cudaGetLastError());
}

template <typename T>
void launch_energy_cot(int ndir, const int* dchi, const long long* msg_off, const T* F, const T* scale, T* C,
                       cudaStream_t s) {
  if (ndir == 0) return;
  energy_cot_kernel<T><<<ndir, 64, 0, s>>>(ndir, dchi, msg_off, F, scale, C);
  GBTN_CUDA(cudaGetLastError());
}

template <typename T>
void launch_energy_terms(int ne, int nterms, const double* coef, const T* t, double* Ee, T* scale, cudaStream_t s) {
  if (ne == 0) return;
  energy_terms_kernel<T><<<(ne + 127) / 128, 128, 0, s>>>(ne, nterms, coef, t, Ee, scale);
  GBTN_CUDA(cudaGetLastError());
}

template void launch_edge_dot<double>(int, const int*, const long long*, const double*, double*, cudaStream_t);
template void launch_edge_dot<zdouble>(int, const int*, const long long*, const zdouble*, zdouble*, cudaStream_t);
template void launch_energy_cot<double>(int, const int*, const long long*, const double*, const double*, double*,
                                        cudaStream_t);
template void launch_energy_cot<zdouble>(int, const int*, const long long*, const zdouble*, const zdouble*,
                                         zdouble*, cudaStream_t);
template void launch_energy_terms<double>(int, int, const double*, const double*, double*, double*, cudaStream_t);
template void launch_energy_terms<zdouble>(int, int, const double*, const zdouble*, double*, zdouble*, cudaStream_t);

void launch_net_sum(int nnet, const int* net_e_ptr, const int* net_e, const double* Ee, double* out, cudaStream_t s) {
  net_sum_kernel<<<nnet, 256, 0, s>>>(net_e_ptr, net_e, Ee, out);
  GBTN_CUDA(cudaGetLastError());
}

void launch_axpy_resid(long long n, const double* a, const double* b, const double* old, double* y, double* acc,
                       cudaStream_t s) {
  GBTN_CUDA(cudaMemsetAsync(acc, 0, 2 * sizeof(double), s));
  long long blocks = (n + 255) / 256;
  if (blocks > 1216) blocks = 1216;
  if (blocks < 1) blocks = 1;
  axpy_resid_kernel<<<(int)blocks, 256, 0, s>>>(n, a, b, old, y, acc);
  GBTN_CUDA(cudaGetLastError());
}

}  // namespace gbtn
