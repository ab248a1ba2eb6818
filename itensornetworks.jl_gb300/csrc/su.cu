// Simple update on the GPU (FP64): apply(o, psi; envs, maxdim, cutoff) for
// two-site gates (simple_update_bp, src/apply.jl:33-95; apply, :97-146), and
// the gate batches of tebd (src/tebd.jl:2-31).
//
// A batch of consecutive gates on disjoint vertices (they commute) runs as
// three launches: su_qr_kernel (one CTA per gate side: steps 1-2),
// su_svd_kernel (one CTA per gate: steps 3-5) and su_rebuild_kernel (one CTA
// per gate side: step 6); complex gates or tensors run the whole gate in one
// CTA (su_gate_z_kernel).  Per gate:
//   1. sqrt / inverse-sqrt of every environment message on the other legs of
//      both sites (Hermitian eigen-decomposition, eigenvalues below 10 eps of
//      the total magnitude dropped -- map_eigvals, apply.jl:9-25);
//   2. each site absorbs its sqrt environments and is QR-factorised as
//      (other legs) x (site, bond) with Householder reflectors: psi = Q R;
//   3. theta = R_u R_v over the bond, the gate applied on the two site indices;
//   4. SVD of theta: pivoted QR, then one-sided Jacobi on R^T (columns
//      rotated in round-robin pairs, eight lanes per pair): sweeps in FP32 to
//      2e-6, a first-order FP64 re-orthogonalisation of their rotation, then
//      FP64 sweeps that skip pairs of noise columns the cutoff discards and
//      stop after a sweep of couplings below 1e-7; singular values sorted in
//      descending order;
//   5. truncation by the rule of ITensors' svd: at most maxdim values, then drop
//      from the tail while the discarded sum of squares stays within
//      cutoff * sum of squares (at least one value kept); truncation error =
//      discarded fraction;
//   6. psi_u = Q_u U sqrt(S), psi_v = Q_v (sqrt(S) V^T)^T, inverse-sqrt
//      environments absorbed back, optional normalisation.
// Site tensors live in fixed-capacity slots (chi_max per leg) holding the
// current shape column-major (site index first); bond dimensions are a device
// array updated by the gate that changes them.
#include <math.h>

#include <algorithm>
#include <memory>
#include <numeric>
#include <vector>

#include "bp_device.cuh"

namespace gbtn {
namespace {

constexpr int kSuThreads = 256;
constexpr int kSuWarps = kSuThreads / 32;
constexpr int kSuMaxN = 8192;     // elements of one site tensor
constexpr int kSuMaxTheta = 64;   // rows / columns of theta
constexpr int kSvdMaxSweeps = 40;
// A Jacobi pair is left alone when its columns are orthogonal to this
// relative precision (a few ulps above the rounding of a 64-long FP64 dot)
// or when either column is below 1e-15 of ||A||_F (rotating rounding noise
// cannot change the decomposition beyond eps ||A||).
constexpr double kJacobiTol = 1e-13;
constexpr double kJacobiTiny = 1e-30;
// A sweep whose rotations all had couplings |g| / sqrt(a b) at or below this
// ends the FP64 Jacobi: each rotation leaves its pair coupled to about 1e-7 of
// its coupling (the FP32 tangent), and later rotations of the sweep couple
// pairs again only by products of two couplings, so every coupling left is
// about 1e-14, below kJacobiTol, and the next sweep would rotate nothing.
constexpr double kJacobiLastSweep = 1e-7;
// Noise bound of the Jacobi stage of a gate's SVD (n singular values, relative
// cutoff on sigma^2): pairs of columns both at or below skip_rel * ||theta||^2
// are not rotated.  Those columns sum to at most n * skip_rel <= cutoff / 2 of
// the total, so the cutoff discards every one of them whatever maxdim did
// first; no cutoff (< 0) or a zero cutoff keeps the full Jacobi.
__host__ __device__ inline double svd_skip_rel(double cutoff, int n) {
  return cutoff > 0.0 ? fmin(1e-16, 0.5 * cutoff / (double)n) : 0.0;
}

// FP64 runs at a small fraction of the FP32 rate on this part, and a warp
// instruction costs the FP64 pipe the same whether one lane or 32 are active,
// so the helpers below keep the number of FP64 warp instructions low: scalar
// work is done by one warp (or one lane) and broadcast through shared memory.

// Sum over the CTA; every thread receives the total.  red: >= kSuWarps + 1.
__device__ __forceinline__ double block_sum(double x, double* red) {
  x = warp_sum(x);
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) red[w] = x;
  __syncthreads();
  if (w == 0) {
    double t = lane < kSuWarps ? red[lane] : 0.0;
#pragma unroll
    for (int o = kSuWarps / 2; o > 0; o >>= 1) t += __shfl_xor_sync(0xffffffffu, t, o);
    if (lane == 0) red[kSuWarps] = t;
  }
  __syncthreads();
  return red[kSuWarps];
}

// Scratch of the SVD: work >= m*n + n*n doubles; cn, rdiag, bet, V-row
// permutation perm and sort order ord >= n entries; flag and red as in
// block_sum; extra >= 2*n*n doubles.
struct SvdBufs {
  double* work;
  double* cn;
  double* rdiag;
  double* bet;
  int* perm;
  int* ord;
  int* flag;
  double* red;
  double* extra;  // >= 2 n^2 doubles: the FP64 re-orthogonalisation of the FP32 rotation
};

// Sum of x over the 8 lanes of a group (all 32 lanes must take part).
__device__ __forceinline__ double group8_sum(double x) {
#pragma unroll
  for (int o = 4; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
  return x;
}

// Householder QR with column pivoting of A (m x n, m >= n, lda = m), in place:
// A P = Q R, column j of A P being column perm[j] of A.  On return the strict
// upper triangle of A holds R, rdiag its diagonal, the columns below the
// diagonal the reflectors (bet their coefficients).  The group that updates a
// column also returns its squared norm below the next row, so the pivot
// norms are exact rather than downdated.
__device__ void cta_qrcp(double* A, int m, int n, SvdBufs& b) {
  __shared__ double s_bj;
  __shared__ int s_piv;
  const int tid = threadIdx.x, grp = tid >> 3, gl = tid & 7, warp = tid >> 5;
  for (int c0 = 0; c0 < n; c0 += 32) {
    const int c = c0 + grp;
    double s2 = 0.0;
    if (c < n)
      for (int i = gl; i < m; i += 8) s2 = fma(A[(size_t)c * m + i], A[(size_t)c * m + i], s2);
    s2 = group8_sum(s2);
    if (c < n && gl == 0) {
      b.cn[c] = s2;
      b.perm[c] = c;
    }
  }
  __syncthreads();
  for (int j = 0; j < n; ++j) {
    if (tid == 0) {  // pivot: largest remaining norm (bit patterns of non-negative doubles order like values)
      int piv = j;
      long long best = __double_as_longlong(b.cn[j]);
      for (int c = j + 1; c < n; ++c) {
        const long long k = __double_as_longlong(b.cn[c]);
        if (k > best) {
          best = k;
          piv = c;
        }
      }
      s_piv = piv;
      if (piv != j) {
        const double t = b.cn[j];
        b.cn[j] = b.cn[piv];
        b.cn[piv] = t;
        const int q = b.perm[j];
        b.perm[j] = b.perm[piv];
        b.perm[piv] = q;
      }
    }
    __syncthreads();
    const int piv = s_piv;
    if (piv != j)
      for (int i = tid; i < m; i += kSuThreads) {
        const double t = A[(size_t)j * m + i];
        A[(size_t)j * m + i] = A[(size_t)piv * m + i];
        A[(size_t)piv * m + i] = t;
      }
    __syncthreads();
    double* x = A + (size_t)j * m;
    if (tid == 0) {
      const double s2 = b.cn[j], x0 = x[j];
      const double nrm = sqrt(s2);
      const double alpha = x0 >= 0.0 ? -nrm : nrm;
      const double v0 = x0 - alpha;
      const double vn2 = s2 - x0 * x0 + v0 * v0;
      const double bj = (vn2 > 0.0 && nrm > 0.0) ? 2.0 / vn2 : 0.0;
      if (bj > 0.0) x[j] = v0;
      b.bet[j] = bj;
      b.rdiag[j] = bj > 0.0 ? alpha : x0;
      s_bj = bj;
    }
    __syncthreads();
    const double bj = s_bj;
    for (int c0 = j + 1; c0 < n; c0 += 32) {
      if (c0 + 4 * warp >= n) continue;  // warp-uniform
      const int c = c0 + grp;
      const bool act = c < n;
      double* y = A + (size_t)(act ? c : j) * m;
      double w = 0.0;
      if (act && bj > 0.0)
        for (int i = j + gl; i < m; i += 8) w = fma(x[i], y[i], w);
      w = group8_sum(w) * bj;
      double nx = 0.0;
      if (act)
        for (int i = j + gl; i < m; i += 8) {
          double v = y[i];
          if (bj > 0.0) {
            v = fma(-w, x[i], v);
            y[i] = v;
          }
          if (i > j) nx = fma(v, v, nx);
        }
      nx = group8_sum(nx);
      if (act && gl == 0) b.cn[c] = nx;
    }
    __syncthreads();
  }
}

// One-sided Jacobi (Hestenes) on the columns of X (m x n, ldx = m).  Columns
// are paired by a round-robin tournament; each pair of a round is handled by
// a group of 8 lanes (32 groups, so a whole round runs at once and one warp
// instruction serves four pairs).  The rotation angle is computed in FP32
// from the FP64 inner products, scaled by the larger norm: it only has to
// shrink the pair's coupling, c^2 + s^2 = 1 is formed in FP64 for whatever
// tangent is used (the transformation stays orthogonal), and the FP64
// stopping test decides the accuracy.  Sweeps stop when a sweep rotates
// nothing.  The rotations are not accumulated: the caller recovers the right
// factor from the rotated columns.  A pair whose squared norms are both at or
// below skip_rel * ||X||_F^2 is left alone: at the end every pair that is not
// orthogonal has both columns below that bound, so a caller whose truncation
// is sure to discard all such columns (n * skip_rel well inside its relative
// cutoff) loses nothing, and the sweeps spent orthogonalising noise columns of
// a rank-deficient theta against each other are saved; skip_rel = 0 keeps
// every column exact.  Sweeps also stop after one whose couplings were all at
// or below kJacobiLastSweep (flag bit 1 marks a larger one).
__device__ void cta_jacobi(double* X, int m, int n, int* flag, double* red, double skip_rel) {
  const int tid = threadIdx.x, grp = tid >> 3, gl = tid & 7;
  double f = 0.0;
  for (int i = tid; i < m * n; i += kSuThreads) f = fma(X[i], X[i], f);
  f = block_sum(f, red);
  const double tiny = f * kJacobiTiny, tol2 = kJacobiTol * kJacobiTol, small = f * skip_rel;
  const double last2 = kJacobiLastSweep * kJacobiLastSweep;
  const int N = n + (n & 1);  // players of the round-robin (one dummy when n is odd)
  const int npair = N / 2;
  const bool warp_busy = (tid >> 5) * 4 < npair;  // warp-uniform
  for (int sweep = 0; sweep < kSvdMaxSweeps; ++sweep) {
    if (tid == 0) *flag = 0;
    __syncthreads();
    for (int r = 0; r < N - 1; ++r) {
      if (warp_busy) {
        int p = 0, q = 0;
        bool act = grp < npair;
        if (act) {
          if (grp == 0) {
            p = N - 1;
            q = r;
          } else {
            p = (r + grp) % (N - 1);
            q = (r - grp + N - 1) % (N - 1);
          }
          if (p > q) {
            const int t = p;
            p = q;
            q = t;
          }
          act = q < n;
        }
        double* a = X + (size_t)p * m;
        double* b = X + (size_t)q * m;
        double al = 0.0, be = 0.0, ga = 0.0;
        if (act)
          for (int i = gl; i < m; i += 8) {
            const double x = a[i], y = b[i];
            al = fma(x, x, al);
            be = fma(y, y, be);
            ga = fma(x, y, ga);
          }
        al = group8_sum(al);
        be = group8_sum(be);
        ga = group8_sum(ga);
        const bool rot = act && al > tiny && be > tiny && fmax(al, be) > small && ga * ga > tol2 * al * be;
        if (__any_sync(0xffffffffu, rot)) {
          // tan of the angle: 2 g sgn(d) / (|d| + sqrt(d^2 + 4 g^2)), d = (be - al) / mx, g = ga / mx
          const float inv = 1.0f / (float)fmax(al, be);
          const float d = (float)(be - al) * inv, g = (float)ga * inv;
          const float t32 = rot ? (d >= 0.f ? 2.f : -2.f) * g / (fabsf(d) + sqrtf(fmaf(d, d, 4.f * g * g))) : 0.f;
          const double t = t32;
          const double c = rsqrt(fma(t, t, 1.0)), s = c * t;
          if (rot) {
            for (int i = gl; i < m; i += 8) {
              const double x = a[i], y = b[i];
              a[i] = fma(c, x, -s * y);
              b[i] = fma(s, x, c * y);
            }
            if (gl == 0) atomicOr(flag, ga * ga > last2 * al * be ? 3 : 1);
          }
        }
      }
      __syncthreads();
    }
    if ((*flag & 2) == 0) break;  // nothing rotated, or only couplings the next sweep would not see
    __syncthreads();
  }
}

// The FP32 stage of the Jacobi SVD: the same tournament on an FP32 copy of
// the columns of X (m x n), rotations accumulated into V (n x n, set to the
// identity here), until a sweep finds every pair orthogonal to 2e-6 (a few
// FP32 roundings above the noise of a 64-long FP32 dot).  Costs the FP64
// pipe nothing; the FP64 stage then starts from nearly orthogonal columns.
__device__ void cta_jacobi32(float* X, int m, int n, float* V, int* flag, double* red) {
  const int tid = threadIdx.x, grp = tid >> 3, gl = tid & 7;
  for (int i = tid; i < n * n; i += kSuThreads) V[i] = (i % n == i / n) ? 1.f : 0.f;
  double f = 0.0;
  for (int i = tid; i < m * n; i += kSuThreads) f += (double)X[i] * (double)X[i];
  f = block_sum(f, red);
  const float tiny = (float)(f * kJacobiTiny), tol2 = 4e-12f;
  const int N = n + (n & 1);
  const int npair = N / 2;
  const bool warp_busy = (tid >> 5) * 4 < npair;
  for (int sweep = 0; sweep < 16; ++sweep) {
    if (tid == 0) *flag = 0;
    __syncthreads();
    for (int r = 0; r < N - 1; ++r) {
      if (warp_busy) {
        int p = 0, q = 0;
        bool act = grp < npair;
        if (act) {
          if (grp == 0) {
            p = N - 1;
            q = r;
          } else {
            p = (r + grp) % (N - 1);
            q = (r - grp + N - 1) % (N - 1);
          }
          if (p > q) {
            const int t = p;
            p = q;
            q = t;
          }
          act = q < n;
        }
        float* a = X + (size_t)p * m;
        float* b = X + (size_t)q * m;
        float al = 0.f, be = 0.f, ga = 0.f;
        if (act)
          for (int i = gl; i < m; i += 8) {
            const float x = a[i], y = b[i];
            al = fmaf(x, x, al);
            be = fmaf(y, y, be);
            ga = fmaf(x, y, ga);
          }
#pragma unroll
        for (int o = 4; o > 0; o >>= 1) {
          al += __shfl_xor_sync(0xffffffffu, al, o);
          be += __shfl_xor_sync(0xffffffffu, be, o);
          ga += __shfl_xor_sync(0xffffffffu, ga, o);
        }
        const bool rot = act && al > tiny && be > tiny && ga * ga > tol2 * al * be;
        if (rot) {
          const float inv = 1.0f / fmaxf(al, be);
          const float d = (be - al) * inv, g = ga * inv;
          const float t = (d >= 0.f ? 2.f : -2.f) * g / (fabsf(d) + sqrtf(fmaf(d, d, 4.f * g * g)));
          const float c = rsqrtf(fmaf(t, t, 1.f)), sn = c * t;
          for (int i = gl; i < m; i += 8) {
            const float x = a[i], y = b[i];
            a[i] = fmaf(c, x, -sn * y);
            b[i] = fmaf(sn, x, c * y);
          }
          float* va = V + (size_t)p * n;
          float* vb = V + (size_t)q * n;
          for (int i = gl; i < n; i += 8) {
            const float x = va[i], y = vb[i];
            va[i] = fmaf(c, x, -sn * y);
            vb[i] = fmaf(sn, x, c * y);
          }
          if (gl == 0) *flag = 1;
        }
      }
      __syncthreads();
    }
    if (*flag == 0) break;
    __syncthreads();
  }
}

// SVD of A (m x n, m >= n, lda = m, n <= 64, m <= 64) by one-sided Jacobi
// preconditioned with a pivoted QR (Drmac and Veselic, SIAM J. Matrix Anal.
// Appl. 29 (2008)): A P = Q R and Jacobi on the columns of X = R^T give
// X W = U_x S, so R = W S U_x^T and A = (A P U_x S^-1) S (P U_x)^T:
// V = P U_x and U = A V S^-1.  The pivoting grades R, which cuts the number
// of sweeps on the wide-range spectra of truncated states.  On return: the
// columns of A hold U (zero where sigma = 0), V (n x n, ldv = n) the right
// singular vectors, sig[n] the singular values, all in descending order of
// sig.  U is accurate to eps ||A|| / sigma per column, which is the accuracy
// of the reconstruction U S V^T that the callers use.  skip_rel is passed to
// the FP64 Jacobi stage (0: every singular triplet exact).
__device__ void cta_svd(double* A, int m, int n, double* V, double* sig, SvdBufs& b, double skip_rel = 0.0) {
  const int tid = threadIdx.x, grp = tid >> 3, gl = tid & 7;
  double* A0 = b.work;                  // m x n copy of the input
  double* X = b.work + (size_t)m * n;   // n x n
  for (int i = tid; i < m * n; i += kSuThreads) A0[i] = A[i];
  __syncthreads();
  cta_qrcp(A, m, n, b);
  for (int i = tid; i < n * n; i += kSuThreads) {  // X[c, r] = R[r, c]
    const int c = i % n, r = i / n;
    X[i] = r < c ? A[(size_t)c * m + r] : (r == c ? b.rdiag[r] : 0.0);
  }
  __syncthreads();
  // FP32 stage on a copy (A's reflectors are no longer needed: X32 and V32
  // live there), then X <- X Q with Q = V32 (I - E / 2), E = V32^T V32 - I,
  // orthonormal to O(|E|^2) = O(1e-14), formed in FP64
  {
    float* X32 = reinterpret_cast<float*>(A);
    float* V32 = X32 + n * n;
    for (int i = tid; i < n * n; i += kSuThreads) X32[i] = (float)X[i];
    __syncthreads();
    cta_jacobi32(X32, n, n, V32, b.flag, b.red);
    double* E = b.extra;
    double* Q = b.extra + (size_t)n * n;
    for (int i = tid; i < n * n; i += kSuThreads) V[i] = (double)V32[i];
    __syncthreads();
    for (int i = tid; i < n * n; i += kSuThreads) {
      const int a = i % n, c = i / n;
      double acc = a == c ? -1.0 : 0.0;
      for (int k = 0; k < n; ++k) acc = fma(V[k + n * a], V[k + n * c], acc);
      E[i] = acc;
    }
    __syncthreads();
    for (int i = tid; i < n * n; i += kSuThreads) {
      const int r = i % n, c = i / n;
      double acc = 0.0;
      for (int k = 0; k < n; ++k) acc = fma(V[r + n * k], E[k + n * c], acc);
      Q[i] = fma(-0.5, acc, V[i]);
    }
    __syncthreads();
    double* XQ = A;
    for (int i = tid; i < n * n; i += kSuThreads) {
      const int r = i % n, c = i / n;
      double acc = 0.0;
      for (int k = 0; k < n; ++k) acc = fma(X[r + n * k], Q[k + n * c], acc);
      XQ[i] = acc;
    }
    __syncthreads();
    for (int i = tid; i < n * n; i += kSuThreads) X[i] = XQ[i];
    __syncthreads();
  }
  cta_jacobi(X, n, n, b.flag, b.red, skip_rel);
  // sigma = column norms of X, U_x = unit columns (a group per column)
  for (int j0 = 0; j0 < n; j0 += 32) {
    const int j = j0 + grp;
    double s2 = 0.0;
    if (j < n)
      for (int i = gl; i < n; i += 8) s2 = fma(X[(size_t)j * n + i], X[(size_t)j * n + i], s2);
    s2 = group8_sum(s2);
    const double sg = sqrt(s2);
    const double iv = sg > 0.0 ? 1.0 / sg : 0.0;
    if (j < n) {
      for (int i = gl; i < n; i += 8) X[(size_t)j * n + i] *= iv;
      if (gl == 0) {
        sig[j] = sg;
        b.cn[j] = iv;
      }
    }
  }
  __syncthreads();
  // V = P U_x: row perm[j] of V is row j of U_x
  for (int i = tid; i < n * n; i += kSuThreads) {
    const int j = i % n, k = i / n;
    V[(size_t)k * n + b.perm[j]] = X[i];
  }
  __syncthreads();
  // U = A V S^-1
  for (int i = tid; i < m * n; i += kSuThreads) {
    const int r = i % m, k = i / m;
    double acc = 0.0;
    for (int c = 0; c < n; ++c) acc = fma(A0[(size_t)c * m + r], V[(size_t)k * n + c], acc);
    A[i] = acc * b.cn[k];
  }
  __syncthreads();
  // descending, stable order by rank counting; sigma >= 0, so the IEEE bit
  // patterns order like the values and the comparisons stay off the FP64 pipe
  if (tid < n) {
    const long long kj = __double_as_longlong(sig[tid]);
    int rank = 0;
    for (int i = 0; i < n; ++i) {
      const long long ki = __double_as_longlong(sig[i]);
      rank += (ki > kj) || (ki == kj && i < tid);
    }
    b.ord[rank] = tid;
  }
  __syncthreads();
  double* U2 = b.work;
  double* V2 = b.work + (size_t)m * n;
  for (int i = tid; i < m * n; i += kSuThreads) U2[i] = A[(size_t)b.ord[i / m] * m + (i % m)];
  for (int i = tid; i < n * n; i += kSuThreads) V2[i] = V[(size_t)b.ord[i / n] * n + (i % n)];
  __syncthreads();
  for (int i = tid; i < m * n; i += kSuThreads) A[i] = U2[i];
  for (int i = tid; i < n * n; i += kSuThreads) V[i] = V2[i];
  __syncthreads();
  if (tid < n) b.work[tid] = sig[b.ord[tid]];
  __syncthreads();
  if (tid < n) sig[tid] = b.work[tid];
  __syncthreads();
}

// Householder QR of M (m x n column-major, lda = m): R (r x n, ldr = r) and
// Q (m x r, ldq = m), r = min(m, n).  M is overwritten by the reflectors
// (column j holds v_j from row j on; beta_j = 0 marks a skipped reflector);
// with Q = NULL the reflectors are the result.  beta: >= n doubles.
// The warp that updates column j + 1 also returns that column's squared norm
// below row j + 1, so each reflector costs two barriers; Q is accumulated
// backwards, touching only the columns a reflector changes.
__device__ void cta_qr(double* M, int m, int n, double* R, double* Q, double* beta, double* red) {
  __shared__ double s_bj, s_next;
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r = m < n ? m : n;
  double s2_first = 0.0;
  for (int i = tid; i < m; i += kSuThreads) s2_first = fma(M[i], M[i], s2_first);
  s2_first = block_sum(s2_first, red);
  for (int j = 0; j < r; ++j) {
    double* x = M + (size_t)j * m;
    if (tid == 0) {
      const double s2 = j == 0 ? s2_first : s_next;
      const double x0 = x[j];
      const double nrm = sqrt(s2);
      const double alpha = x0 >= 0.0 ? -nrm : nrm;
      const double v0 = x0 - alpha;
      const double vn2 = s2 - x0 * x0 + v0 * v0;
      const double bj = (vn2 > 0.0 && nrm > 0.0) ? 2.0 / vn2 : 0.0;
      if (bj > 0.0) x[j] = v0;  // the reflector v occupies x[j..m)
      beta[j] = bj;
      R[j + (size_t)r * j] = bj > 0.0 ? alpha : x0;
      s_bj = bj;
    }
    __syncthreads();
    const double bj = s_bj;
    for (int c = j + 1 + warp; c < n; c += kSuWarps) {
      double* y = M + (size_t)c * m;
      double w = 0.0;
      if (bj > 0.0) {
        for (int i = j + lane; i < m; i += 32) w = fma(x[i], y[i], w);
        w = warp_sum(w) * bj;
      }
      double nx = 0.0;
      for (int i = j + lane; i < m; i += 32) {
        double v = y[i];
        if (bj > 0.0) {
          v = fma(-w, x[i], v);
          y[i] = v;
        }
        if (c == j + 1 && i > j) nx = fma(v, v, nx);
      }
      if (c == j + 1) {
        nx = warp_sum(nx);
        if (lane == 0) s_next = nx;
      }
    }
    __syncthreads();
  }
  // R: upper triangle (diagonal set above), rest from M
  for (int i = tid; i < r * n; i += kSuThreads) {
    const int row = i % r, col = i / r;
    if (col > row) R[i] = M[(size_t)col * m + row];
    else if (col < row) R[i] = 0.0;
  }
  if (!Q) {  // the caller keeps the reflectors and applies them itself
    __syncthreads();
    return;
  }
  // Q = H_0 ... H_{r-1} [I; 0]; H_j leaves the columns c < j (still e_c) alone
  for (int i = tid; i < m * r; i += kSuThreads) Q[i] = (i % m == i / m) ? 1.0 : 0.0;
  __syncthreads();
  for (int j = r - 1; j >= 0; --j) {
    const double bj = beta[j];
    if (bj == 0.0) continue;
    const double* x = M + (size_t)j * m;
    for (int c = j + warp; c < r; c += kSuWarps) {
      double* y = Q + (size_t)c * m;
      double w = 0.0;
      for (int i = j + lane; i < m; i += 32) w = fma(x[i], y[i], w);
      w = warp_sum(w) * bj;
      for (int i = j + lane; i < m; i += 32) y[i] = fma(-w, x[i], y[i]);
    }
    __syncthreads();
  }
}

// sqrt(env) and inverse sqrt(env) of a symmetric chi x chi message through its
// eigen-decomposition (the singular vectors of a positive semi-definite
// matrix), dropping the smallest eigenvalues while their summed magnitude is
// within 10 eps of the total.  S, Si: chi x chi column-major.
__device__ void cta_env_sqrt(const double* env, int chi, double* S, double* Si, double* A, double* V, double* sig,
                             SvdBufs& sb) {
  const int tid = threadIdx.x;
  for (int i = tid; i < chi * chi; i += kSuThreads) {
    const int b = i % chi, a = i / chi;
    A[i] = 0.5 * (env[b + chi * a] + env[a + chi * b]);
  }
  __syncthreads();
  cta_svd(A, chi, chi, V, sig, sb);
  __shared__ int s_keep;
  if (tid == 0) {
    double tot = 0.0;
    for (int j = 0; j < chi; ++j) tot += sig[j];
    if (tot == 0.0) tot = 1.0;
    int k = chi;
    double disc = 0.0;
    while (k > 1 && disc + sig[k - 1] <= 10.0 * 2.220446049250313e-16 * tot) {
      disc += sig[k - 1];
      --k;
    }
    s_keep = k;
  }
  __syncthreads();
  const int k = s_keep;
  double* rs = sb.work;       // sqrt of the kept eigenvalues
  double* ri = sb.work + 64;  // and their inverses
  if (tid < k) {
    const double q = sqrt(sig[tid]);
    rs[tid] = q;
    ri[tid] = 1.0 / q;
  }
  __syncthreads();
  for (int i = tid; i < chi * chi; i += kSuThreads) {
    const int b = i % chi, a = i / chi;
    double s = 0.0, si = 0.0;
    for (int j = 0; j < k; ++j) {
      const double vv = V[b + chi * j] * V[a + chi * j];
      s = fma(vv, rs[j], s);
      si = fma(vv, ri[j], si);
    }
    S[i] = s;
    Si[i] = si;
  }
  __syncthreads();
}

}  // namespace
}  // namespace gbtn

namespace gbtn {
namespace {

struct SuJob {
  int e, u, v, pu, pv;
};

struct SuArgs {
  const SuJob* jobs;
  int njobs;
  const int* leg_ptr;
  const int* leg_edge;
  const int* edge_u;
  const int* site_dim;
  int* edim;                 // current bond dimensions (updated)
  const long long* cap_off;  // slot of every vertex
  double* tens;              // capacity storage
  const double* envs;        // NULL or 2*ne messages of chi_max^2 each (compact chi x chi)
  const double* gates;
  long long gate_stride;     // 0: one gate for all jobs
  int maxdim;
  double cutoff;
  int normalize;
  int chimax;
  double* side_scratch;      // per (job, side): reflectors, beta, R, inverse-sqrt environments, rank
  double* job_scratch;       // per job: left / right factors, sqrt(S), kept dimension
  int bmax;                  // bound on theta's rows and columns (shared-memory carve of the SVD)
  double* truncerr;          // [njobs] or NULL
  double* svals;             // [njobs * maxdim] or NULL
  int* status;               // set to 1 when a shape exceeds the kernel limits
  // adjoint runs only (NULL otherwise): the full SVD of theta per job and the
  // square-root environments per (job, side), written by the forward stages
  double* svd_full;
  double* side_sqrt;
};

struct SideShape {
  int d, k, n, p;   // site dim, links, elements, leg of the bond
  int chi[kMaxDeg];
  int m;            // product of the other legs' dims
};

__device__ void side_shape(const SuArgs& a, int x, int p, SideShape& sh) {
  sh.d = a.site_dim[x];
  sh.k = a.leg_ptr[x + 1] - a.leg_ptr[x];
  sh.p = p;
  int n = sh.d, m = 1;
  for (int q = 0; q < sh.k; ++q) {
    sh.chi[q] = a.edim[a.leg_edge[a.leg_ptr[x] + q]];
    n *= sh.chi[q];
    if (q != p) m *= sh.chi[q];
  }
  sh.n = n;
  sh.m = m;
}

// element idx of a tensor with dims (d, chi[0..k)) -> (row over the other legs, site s, bond index)
__device__ __forceinline__ void split_index(const SideShape& sh, const int* chi, int idx, int& row, int& s, int& b) {
  s = idx % sh.d;
  int rest = idx / sh.d, rs = 1;
  row = 0;
  b = 0;
  for (int q = 0; q < sh.k; ++q) {
    const int l = rest % chi[q];
    rest /= chi[q];
    if (q == sh.p) {
      b = l;
    } else {
      row += l * rs;
      rs *= chi[q];
    }
  }
}

// Scratch between the three stages of a gate batch (global memory).
constexpr int kSideRefl = 0;                           // m x r reflectors, lda = m
constexpr int kSideBeta = kSuMaxN;                     // r reflector coefficients
constexpr int kSideR = kSideBeta + 64;                 // r x ncol, ldr = r
constexpr int kSideSI = kSideR + 2048;                 // inverse-sqrt environments, kMaxDeg x 64
constexpr int kSideMeta = kSideSI + kMaxDeg * 64;      // [0] = r, [1] = status
constexpr int kSideStride = kSideMeta + 8;
constexpr int kJobU = 0;                               // left factor, mt x kk (ld mt)
constexpr int kJobV = kSuMaxTheta * kSuMaxTheta;       // right factor, nt x kk (ld nt)
constexpr int kJobS = 2 * kSuMaxTheta * kSuMaxTheta;   // sqrt of the kept singular values
constexpr int kJobMeta = kJobS + kSuMaxTheta;          // [0] = kk, [1] = ok
constexpr int kJobStride = kJobMeta + 8;
constexpr int kFullU = 0;                              // all left singular vectors, mt x n (ld mt)
constexpr int kFullV = kSuMaxTheta * kSuMaxTheta;      // all right singular vectors, nt x n (ld nt)
constexpr int kFullSig = 2 * kSuMaxTheta * kSuMaxTheta;  // all n singular values, descending
constexpr int kFullStride = kFullSig + kSuMaxTheta;
constexpr int kSqrtStride = kMaxDeg * 64;              // sqrt environment of every leg, chi x chi

// The gate's site on `side`: shape with the current bond dimensions, and
// whether the stages' limits hold (uniform over the CTA).
__device__ bool site_of(const SuArgs& a, const SuJob& job, int side, int& x, SideShape& h) {
  x = side ? job.v : job.u;
  side_shape(a, x, side ? job.pv : job.pu, h);
  const int ce = h.chi[h.p];
  const int r = min(h.m, h.d * ce);
  // the rebuilt site (bond up to maxdim) must fit the same buffers
  return h.n <= kSuMaxN && h.n / ce * max(a.maxdim, ce) <= kSuMaxN && h.d * ce <= 32 && h.k <= kMaxDeg &&
         r * h.d <= a.bmax;
}

// Stage 1, one CTA per (gate, side): square-root environments absorbed,
// the site matricised as (other legs) x (site, bond) and QR-factorised
// (Householder, Q kept as reflectors).  Writes R, the reflectors, beta and
// the inverse-square-root environments to the side's scratch.
__global__ void __launch_bounds__(kSuThreads, 3) su_qr_kernel(SuArgs a) {
  extern __shared__ __align__(16) double smem[];
  const int j = blockIdx.x >> 1, side = blockIdx.x & 1, tid = threadIdx.x;
  if (j >= a.njobs) return;
  const SuJob job = a.jobs[j];
  int x;
  SideShape h;
  const bool ok = site_of(a, job, side, x, h);
  double* out = a.side_scratch + (size_t)blockIdx.x * kSideStride;
  if (!ok) {
    if (tid == 0) {
      atomicExch(a.status, 1);
      out[kSideMeta + 1] = 1.0;
    }
    return;
  }
  double* W = smem;                       // matricised site (then reflectors), kSuMaxN
  double* T = W + kSuMaxN;                // site tensor when environments are absorbed, kSuMaxN
  double* small = T + (a.envs ? kSuMaxN : 0);
  double* R = small;                      // 1024
  double* beta = R + 1024;                // 64
  double* red = beta + 64;                // 32
  double* S = red + 32;                   // 64
  double* A8 = S + 64;                    // 64: environment matrix
  double* V8 = A8 + 64;                   // 64
  double* sig = V8 + 64;                  // 64
  double* aux = sig + 64;                 // 192
  int* ord = reinterpret_cast<int*>(aux + 192);  // 64
  int* perm = ord + 64;                   // 64
  __shared__ int s_flag;
  const double* src = a.tens + a.cap_off[x];
  const int ce = h.chi[h.p], ncol = h.d * ce;
  if (a.envs) {
    SvdBufs sb{W, aux, aux + 64, aux + 128, perm, ord, &s_flag, red, nullptr};
    for (int i = tid; i < h.n; i += kSuThreads) T[i] = src[i];
    __syncthreads();
    double* cur = T;
    double* nxt = W;
    int st = h.d;
    for (int q = 0; q < h.k; ++q) {
      if (q != h.p) {
        const int f = a.leg_edge[a.leg_ptr[x] + q];
        const int de_in = a.edge_u[f] == x ? 2 * f + 1 : 2 * f;
        const double* env = a.envs + (size_t)de_in * a.chimax * a.chimax;
        sb.work = nxt;                   // free here: m n + n^2 <= 128 doubles used
        sb.extra = nxt + kSuMaxN / 2;    // 2 n^2 <= 128 doubles
        cta_env_sqrt(env, h.chi[q], S, out + kSideSI + q * 64, A8, V8, sig, sb);
        if (a.side_sqrt)
          for (int i = tid; i < h.chi[q] * h.chi[q]; i += kSuThreads)
            a.side_sqrt[(size_t)blockIdx.x * kSqrtStride + q * 64 + i] = S[i];
        absorb_any<double>(h.chi[q], cur, nxt, h.n, st, S, tid, kSuThreads);
        __syncthreads();
        double* t = cur;
        cur = nxt;
        nxt = t;
      }
      st *= h.chi[q];
    }
    if (cur == W) {  // the matricised copy goes to W
      for (int i = tid; i < h.n; i += kSuThreads) T[i] = W[i];
      __syncthreads();
    }
    for (int i = tid; i < h.n; i += kSuThreads) {
      int row, s, b;
      split_index(h, h.chi, i, row, s, b);
      W[row + (size_t)h.m * (s + h.d * b)] = T[i];
    }
  } else {
    for (int i = tid; i < h.n; i += kSuThreads) {
      int row, s, b;
      split_index(h, h.chi, i, row, s, b);
      W[row + (size_t)h.m * (s + h.d * b)] = src[i];
    }
  }
  __syncthreads();
  const int r = min(h.m, ncol);
  cta_qr(W, h.m, ncol, R, nullptr, beta, red);
  for (int i = tid; i < h.m * r; i += kSuThreads) out[kSideRefl + i] = W[i];
  for (int i = tid; i < r * ncol; i += kSuThreads) out[kSideR + i] = R[i];
  if (tid < r) out[kSideBeta + tid] = beta[tid];
  if (tid == 0) {
    out[kSideMeta] = (double)r;
    out[kSideMeta + 1] = 0.0;
  }
}

// Stage 2, one CTA per gate: theta = R_u R_v over the bond with the gate on
// the two site indices, its SVD and the ITensors truncation.  Writes the kept
// left and right factors, sqrt(S) and the new bond dimension.
__global__ void __launch_bounds__(kSuThreads, 2) su_svd_kernel(SuArgs a) {
  extern __shared__ __align__(16) double smem[];
  const int j = blockIdx.x, tid = threadIdx.x;
  if (j >= a.njobs) return;
  const SuJob job = a.jobs[j];
  const double* su = a.side_scratch + (size_t)(2 * j) * kSideStride;
  const double* sv = a.side_scratch + (size_t)(2 * j + 1) * kSideStride;
  double* out = a.job_scratch + (size_t)j * kJobStride;
  if (su[kSideMeta + 1] != 0.0 || sv[kSideMeta + 1] != 0.0) {  // a side exceeded the limits
    if (tid == 0) out[kJobMeta + 1] = 0.0;
    return;
  }
  const int B = a.bmax;
  double* TH = smem;                      // B x B
  double* V = TH + B * B;                 // B x B
  double* W = V + B * B;                  // 2 B x B (theta build, SVD work)
  double* RU = W + 2 * B * B;             // 1024
  double* RV = RU + 1024;                 // 1024
  double* XT = RV + 1024;                 // 2 B x B: FP64 re-orthogonalisation in the SVD
  double* sig = XT + 2 * B * B;           // 64
  double* red = sig + 64;                 // 32
  double* aux = red + 32;                 // 192
  int* ord = reinterpret_cast<int*>(aux + 192);  // 64
  int* perm = ord + 64;                   // 64
  __shared__ int s_flag, s_k;
  int xu, xv;
  SideShape hu, hv;
  site_of(a, job, 0, xu, hu);
  site_of(a, job, 1, xv, hv);
  const int ce = hu.chi[hu.p];
  const int du = hu.d, dv = hv.d, ru = (int)su[kSideMeta], rv = (int)sv[kSideMeta];
  for (int i = tid; i < ru * du * ce; i += kSuThreads) RU[i] = su[kSideR + i];
  for (int i = tid; i < rv * dv * ce; i += kSuThreads) RV[i] = sv[kSideR + i];
  __syncthreads();
  // theta[(ru, su), (sv, rv)] = sum_e Ru[ru, su + du e] Rv[rv, sv + dv e], then the gate
  const int mt = ru * du, nt = dv * rv;
  for (int i = tid; i < mt * nt; i += kSuThreads) {
    const int row = i % mt, col = i / mt;
    const int iu = row % ru, su_ = row / ru, sv_ = col % dv, iv = col / dv;
    double acc = 0.0;
    for (int e = 0; e < ce; ++e) acc = fma(RU[iu + ru * (su_ + du * e)], RV[iv + rv * (sv_ + dv * e)], acc);
    W[i] = acc;
  }
  __syncthreads();
  const double* G = a.gates + (size_t)a.gate_stride * j;
  const int D = du * dv;
  for (int i = tid; i < mt * nt; i += kSuThreads) {
    const int row = i % mt, col = i / mt;
    const int iu = row % ru, spu = row / ru, spv = col % dv, iv = col / dv;
    double acc = 0.0;
    for (int sv_ = 0; sv_ < dv; ++sv_)
      for (int su_ = 0; su_ < du; ++su_)
        acc = fma(G[(spu + du * spv) + D * (su_ + du * sv_)], W[(iu + ru * su_) + mt * (sv_ + dv * iv)], acc);
    TH[i] = acc;
  }
  __syncthreads();
  // the SVD wants rows >= columns: a wide theta is decomposed transposed, and
  // its factors swap roles (U of theta^T is V of theta)
  const bool wide = mt < nt;
  if (wide) {
    for (int i = tid; i < mt * nt; i += kSuThreads) W[(i / mt) + nt * (i % mt)] = TH[i];
    __syncthreads();
    for (int i = tid; i < mt * nt; i += kSuThreads) TH[i] = W[i];
    __syncthreads();
  }
  SvdBufs sb{W, aux, aux + 64, aux + 128, perm, ord, &s_flag, red, XT};
  cta_svd(TH, wide ? nt : mt, wide ? mt : nt, V, sig, sb, svd_skip_rel(a.cutoff, min(mt, nt)));
  const double* UF = wide ? V : TH;  // left factor, mt x nsv (ld mt)
  const double* VF = wide ? TH : V;  // right factor, nt x nsv (ld nt)
  if (tid == 0) {
    // ITensors truncation of p = sigma^2 (descending): maxdim, then relative cutoff
    const int nsv = min(mt, nt);
    int n = nsv;
    double te = 0.0, scale = 0.0;
    for (int i = 0; i < nsv; ++i) scale += sig[i] * sig[i];
    if (a.maxdim > 0)
      while (n > a.maxdim) {
        te += sig[n - 1] * sig[n - 1];
        --n;
      }
    if (scale == 0.0) scale = 1.0;
    if (a.cutoff >= 0.0)
      while (n > 1 && te + sig[n - 1] * sig[n - 1] <= a.cutoff * scale) {
        te += sig[n - 1] * sig[n - 1];
        --n;
      }
    if (n < 1) n = 1;
    s_k = n;
    if (a.truncerr) a.truncerr[j] = te / scale;
    if (a.svals)
      for (int i = 0; i < a.maxdim; ++i) a.svals[(size_t)j * a.maxdim + i] = i < n ? sig[i] : 0.0;
    out[kJobMeta] = (double)n;
    out[kJobMeta + 1] = 1.0;
    a.edim[job.e] = n;
  }
  __syncthreads();
  const int kk = s_k;
  if (a.svd_full) {
    const int nsv = min(mt, nt);
    double* full = a.svd_full + (size_t)j * kFullStride;
    for (int i = tid; i < mt * nsv; i += kSuThreads) full[kFullU + i] = UF[i];
    for (int i = tid; i < nt * nsv; i += kSuThreads) full[kFullV + i] = VF[i];
    if (tid < nsv) full[kFullSig + tid] = sig[tid];
  }
  for (int i = tid; i < mt * kk; i += kSuThreads) out[kJobU + i] = UF[i];
  for (int i = tid; i < nt * kk; i += kSuThreads) out[kJobV + i] = VF[i];
  if (tid < kk) out[kJobS + tid] = sqrt(sig[tid]);  // sqrt(S), split onto both sites
}

// Y (m x ncol, ld m) <- Q Y = H_0 ... H_{r-1} Y, or Q^T Y = H_{r-1} ... H_0 Y
// with transpose (each H_j = I - beta_j v_j v_j^T is symmetric), with the
// reflectors of a side's scratch: v_j in rows j..m of column j (beta_j = 0:
// skipped).  Ends with a CTA barrier.
__device__ void apply_reflectors(const double* ss, int m, int r, double* Y, int ncol, bool transpose) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int t = 0; t < r; ++t) {
    const int jr = transpose ? t : r - 1 - t;
    const double bj = ss[kSideBeta + jr];
    if (bj == 0.0) continue;
    const double* v = ss + kSideRefl + (size_t)jr * m;
    for (int c = warp; c < ncol; c += kSuWarps) {
      double* y = Y + (size_t)c * m;
      double w = 0.0;
      for (int i = jr + lane; i < m; i += 32) w = fma(v[i], y[i], w);
      w = warp_sum(w) * bj;
      for (int i = jr + lane; i < m; i += 32) y[i] = fma(-w, v[i], y[i]);
    }
    __syncthreads();
  }
}

// Stage 3, one CTA per (gate, side): the new site = Q (U sqrt(S)) (or
// Q (V sqrt(S)) on the right), Q applied as its reflectors, rearranged to
// the tensor layout with the new bond dimension, inverse-sqrt environments
// absorbed back, optionally normalised, written to the site's slot.
__global__ void __launch_bounds__(kSuThreads, 3) su_rebuild_kernel(SuArgs a) {
  extern __shared__ __align__(16) double smem[];
  const int j = blockIdx.x >> 1, side = blockIdx.x & 1, tid = threadIdx.x;
  if (j >= a.njobs) return;
  const double* js = a.job_scratch + (size_t)j * kJobStride;
  if (js[kJobMeta + 1] == 0.0) return;  // the gate exceeded the limits (status already set)
  const SuJob job = a.jobs[j];
  const double* ss = a.side_scratch + (size_t)blockIdx.x * kSideStride;
  double* Y = smem;                       // m x (d kk), then the tensor
  double* T = Y + kSuMaxN;                // second buffer when environments are absorbed
  double* small = T + (a.envs ? kSuMaxN : 0);
  double* S = small;                      // 64
  double* red = S + 64;                   // 32
  __shared__ double s_scale;
  const int kk = (int)js[kJobMeta];
  // shape: the other legs as before (edim of this gate's bond already holds kk)
  SideShape h;
  const int x = side ? job.v : job.u;
  side_shape(a, x, side ? job.pv : job.pu, h);
  int chi2[kMaxDeg];
  for (int q = 0; q < h.k; ++q) chi2[q] = h.chi[q];
  chi2[h.p] = kk;
  const int m = h.m, d = h.d, ncol2 = d * kk;
  int n2 = d;
  for (int q = 0; q < h.k; ++q) n2 *= chi2[q];
  const int r = (int)ss[kSideMeta];
  // X = U sqrt(S) (rows t, columns s + d b) in the top r rows of Y, zeros below
  const int du = a.site_dim[job.u], dv = a.site_dim[job.v];
  const int ru = (int)a.side_scratch[(size_t)(2 * j) * kSideStride + kSideMeta];
  const int rv = (int)a.side_scratch[(size_t)(2 * j + 1) * kSideStride + kSideMeta];
  const int mt = ru * du, nt = dv * rv;
  for (int i = tid; i < m * ncol2; i += kSuThreads) {
    const int row = i % m, col = i / m, s = col % d, b = col / d;
    double v = 0.0;
    if (row < r)
      v = side == 0 ? js[kJobU + (row + ru * s) + (size_t)mt * b] * js[kJobS + b]
                    : js[kJobV + (s + dv * row) + (size_t)nt * b] * js[kJobS + b];
    Y[i] = v;
  }
  __syncthreads();
  apply_reflectors(ss, m, r, Y, ncol2, false);
  double* dst = a.tens + a.cap_off[x];
  if (a.envs) {
    // tensor layout into T, then the inverse-sqrt environments (T <-> Y)
    for (int i = tid; i < n2; i += kSuThreads) {
      int row, s, b;
      split_index(h, chi2, i, row, s, b);
      T[i] = Y[row + (size_t)m * (s + d * b)];
    }
    __syncthreads();
    double* cur = T;
    double* nxt = Y;
    int st = d;
    for (int q = 0; q < h.k; ++q) {
      if (q != h.p) {
        const int c = chi2[q];
        const double* si = ss + kSideSI + q * 64;
        for (int i = tid; i < c * c; i += kSuThreads) S[(i / c) + c * (i % c)] = si[i];  // transpose
        __syncthreads();
        absorb_any<double>(c, cur, nxt, n2, st, S, tid, kSuThreads);
        __syncthreads();
        double* t = cur;
        cur = nxt;
        nxt = t;
      }
      st *= chi2[q];
    }
    double s2 = 0.0;
    if (a.normalize)
      for (int i = tid; i < n2; i += kSuThreads) s2 = fma(cur[i], cur[i], s2);
    s2 = block_sum(s2, red);
    if (tid == 0) s_scale = (a.normalize && s2 > 0.0) ? 1.0 / sqrt(s2) : 1.0;
    __syncthreads();
    for (int i = tid; i < n2; i += kSuThreads) dst[i] = cur[i] * s_scale;
  } else {
    // the permutation to the tensor layout keeps the norm: normalise from Y
    double s2 = 0.0;
    if (a.normalize)
      for (int i = tid; i < m * ncol2; i += kSuThreads) s2 = fma(Y[i], Y[i], s2);
    s2 = block_sum(s2, red);
    if (tid == 0) s_scale = (a.normalize && s2 > 0.0) ? 1.0 / sqrt(s2) : 1.0;
    __syncthreads();
    for (int i = tid; i < n2; i += kSuThreads) {
      int row, s, b;
      split_index(h, chi2, i, row, s, b);
      dst[i] = Y[row + (size_t)m * (s + d * b)] * s_scale;
    }
  }
}

// ---------------------------------------------------------------------------
// Adjoint of a gate batch (real FP64).  The forward stages have left, per
// job, the reflectors Q, R, beta and the inverse-sqrt environments of both
// sides, the full SVD theta = U diag(sigma) V^T (n = min(mt, nt) values,
// descending), the kept dimension k and the square-root environments.  With
// W_x = Q_x R_x the matricised site (sqrt environments absorbed) and P_x =
// Q_x (x) 1_site, the outputs are the two halves L = P_u U_k sqrt(sigma_k),
// R = P_v V_k sqrt(sigma_k) of the truncated SVD of Theta = P_u theta P_v^T,
// inverse-sqrt environments absorbed, optionally normalised.  Given their
// cotangents:
//   1. normalisation and environment absorption backwards (both linear maps of
//      symmetric matrices, transposed);
//   2. the cotangents of L and R split into their parts in range(P_x)
//      (Z = Q^T Ybar) and orthogonal to it (Ybar_perp);
//   3. the truncated-SVD adjoint in range(P_u) x range(P_v) (Townsend 2016,
//      "Differentiating the singular value decomposition", with the
//      discarded singular values of theta in F_ij = 1/(sigma_j^2 - sigma_i^2)
//      and zero cotangents on the discarded vectors):
//        thetabar = U [F o (U^T Ubar - Ubar^T U) S + diag(sigmabar)
//                      + S F o (V^T Vbar - Vbar^T V)] V^T
//                   + (1 - U U^T) Ubar S_k^-1 V_k^T + U_k S_k^-1 Vbar^T (1 - V V^T);
//      the parts orthogonal to range(P_x) add Ubar_perp S_k^-1 (P_v V_k)^T and
//      (P_u U_k) S_k^-1 Vbar_perp^T, whose contraction with the other site
//      only sees R of that site (Q^T Q = 1) and nothing of its own R;
//   4. through the gate (its transpose) and the bond contraction to Rbar_x,
//      Wbar_x = Q_x Rbar_x + the orthogonal term, then the square-root
//      environments backwards to the cotangent of the site tensor.
// The gate's cotangent is <thetabar, theta_pre> over the row and column
// indices.  Environments are constants.  Pairs of singular values closer
// than 1e-14 sigma_max^2 (degenerate) get F = 0, and kept singular values at
// zero give no derivative (S_k^-1 as a pseudo-inverse).
// ---------------------------------------------------------------------------

constexpr int kVjpSmall = kSuMaxTheta * kSuMaxTheta;  // 4096
// per side
constexpr int kVjY = 0;                     // Ybar (m x d k), then its part orthogonal to range(Q)
constexpr int kVjT0 = kVjY + kSuMaxN;       // tensor ping
constexpr int kVjT1 = kVjT0 + kSuMaxN;      // tensor pong
constexpr int kVjW = kVjT1 + kSuMaxN;       // Wbar (m x d chi)
constexpr int kVjZ = kVjW + kSuMaxN;        // Z = Q^T Ybar (r x d k)
constexpr int kVjRb = kVjZ + kVjpSmall;     // Rbar (r x d chi)
constexpr int kVjH = kVjRb + kVjpSmall;     // H (d k x d chi)
constexpr int kVjM = kVjH + kVjpSmall;      // M (k x d x d chi)
constexpr int kVjChainC = kVjM + kVjpSmall;  // Y and its inverse-sqrt-absorbed stages (kMaxDeg tensors)
constexpr int kVjChainB = kVjChainC + kMaxDeg * kSuMaxN;  // A and its sqrt-absorbed stages
constexpr int kVjSiBar = kVjChainB + kMaxDeg * kSuMaxN;   // dL/d(inverse sqrt environment), per leg
constexpr int kVjSBar = kVjSiBar + kMaxDeg * 64;          // dL/d(sqrt environment), per leg
constexpr int kVjSide = kVjSBar + kMaxDeg * 64;
// per job, after both sides
constexpr int kVjUb = 2 * kVjSide;          // Ubar in range (mt x k)
constexpr int kVjVb = kVjUb + kVjpSmall;    // Vbar in range (nt x k)
constexpr int kVjUtUb = kVjVb + kVjpSmall;  // U^T Ubar (n x k)
constexpr int kVjVtVb = kVjUtUb + kVjpSmall;
constexpr int kVjJ = kVjVtVb + kVjpSmall;   // n x n
constexpr int kVjUJ = kVjJ + kVjpSmall;     // U J (mt x n)
constexpr int kVjP1 = kVjUJ + kVjpSmall;    // (1 - U U^T) Ubar S^-1 (mt x k)
constexpr int kVjP2 = kVjP1 + kVjpSmall;    // (1 - V V^T) Vbar S^-1 (nt x k)
constexpr int kVjTb = kVjP2 + kVjpSmall;    // thetabar (mt x nt)
constexpr int kVjPhi = kVjTb + kVjpSmall;   // gate^T thetabar (mt x nt)
constexpr int kVjPsi = kVjPhi + kVjpSmall;  // theta before the gate (mt x nt)
constexpr int kVjSb = kVjPsi + kVjpSmall;   // sigmabar, each side's part (2 x kSuMaxTheta)
constexpr int kVjStride = kVjSb + 2 * kSuMaxTheta;  // sigmabar: one part per side

__device__ __forceinline__ double safe_inv(double x) { return x > 0.0 ? 1.0 / x : 0.0; }

// R[b + c a] = sum over the fibers of leg (st, c) of X[.. b ..] Y[.. a ..]
// (n elements): the cotangent of the matrix M of an absorption
// out[.. b ..] = sum_a M[b + c a] in[.. a ..], with X = dL/d(out), Y = in.
// One warp per entry; ends with a CTA barrier.
__device__ void leg_gram(const double* X, const double* Y, int n, int st, int c, double* R) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nfib = n / c;
  for (int o = warp; o < c * c; o += kSuWarps) {
    const int b = o % c, a_ = o / c;
    double acc = 0.0;
    for (int f = lane; f < nfib; f += 32) {
      const int lo = f % st, base = lo + (f - lo) * c;
      acc = fma(X[base + b * st], Y[base + a_ * st], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) R[o] = acc;
  }
  __syncthreads();
}

// The per-gate context of the three adjoint launches.
struct VjpCtx {
  SuJob job;
  const double* ssd[2];  // the sides' scratch of the forward's QR stage
  const double* js;      // the job's scratch of the forward's SVD stage
  SideShape hs[2];
  int xs[2];
  int k, ce, du, dv, D, ru, rv, mt, nt, n;
  double* wj;
};

// False when the gate is skipped: a forward stage exceeded its limits (status
// already set) or the recomputed truncation differs from post_dims (status 2).
__device__ bool vjp_ctx(const SuArgs& a, const int* post_dims, double* work, int j, VjpCtx& c) {
  c.job = a.jobs[j];
  c.ssd[0] = a.side_scratch + (size_t)(2 * j) * kSideStride;
  c.ssd[1] = a.side_scratch + (size_t)(2 * j + 1) * kSideStride;
  c.js = a.job_scratch + (size_t)j * kJobStride;
  if (c.ssd[0][kSideMeta + 1] != 0.0 || c.ssd[1][kSideMeta + 1] != 0.0 || c.js[kJobMeta + 1] == 0.0) return false;
  c.k = (int)c.js[kJobMeta];
  if (c.k != post_dims[c.job.e]) {
    if (threadIdx.x == 0) atomicExch(a.status, 2);
    return false;
  }
  site_of(a, c.job, 0, c.xs[0], c.hs[0]);
  site_of(a, c.job, 1, c.xs[1], c.hs[1]);
  c.ce = c.hs[0].chi[c.hs[0].p];
  c.du = c.hs[0].d;
  c.dv = c.hs[1].d;
  c.D = c.du * c.dv;
  c.ru = (int)c.ssd[0][kSideMeta];
  c.rv = (int)c.ssd[1][kSideMeta];
  c.mt = c.ru * c.du;
  c.nt = c.dv * c.rv;
  c.n = min(c.mt, c.nt);
  c.wj = work + (size_t)j * kVjStride;
  return true;
}

// Stage 1, one CTA per (gate, side): the forward's output rebuilt for the
// normalisation, normalisation and inverse-sqrt environments backwards, the
// cotangent split into Z = Q^T Ybar and Ybar_perp, the in-range cotangents of
// the singular vectors and this side's part of sigmabar.
__global__ void __launch_bounds__(kSuThreads, 2)
    su_vjp_side_kernel(SuArgs a, const int* post_dims, const double* cot_out, double* work, int want_env) {
  const int j = blockIdx.x >> 1, side = blockIdx.x & 1, tid = threadIdx.x;
  if (j >= a.njobs) return;
  __shared__ double red[kSuWarps + 1];
  __shared__ double s_scale, s_dot;
  VjpCtx c;
  if (!vjp_ctx(a, post_dims, work, j, c)) return;
  const double* ssd[2] = {c.ssd[0], c.ssd[1]};
  const SideShape* hs = c.hs;
  const int* xs = c.xs;
  const int k = c.k, ru = c.ru, dv = c.dv, mt = c.mt, nt = c.nt;
  const double* js = c.js;
  const double* full = a.svd_full + (size_t)j * kFullStride;
  const double* UF = full + kFullU;
  const double* VF = full + kFullV;
  double* wj = c.wj;
  double* Ub = wj + kVjUb;
  double* Vb = wj + kVjVb;
  double* sb = wj + kVjSb;
  const SideShape& h = hs[side];
  const double* ss = ssd[side];
  double* ws = wj + (size_t)side * kVjSide;
  double* Y = ws + kVjY;
  double* Z = ws + kVjZ;
  const int x = xs[side], m = h.m, d = h.d, r = (int)ss[kSideMeta];
  int chi2[kMaxDeg];
  for (int q = 0; q < h.k; ++q) chi2[q] = h.chi[q];
  chi2[h.p] = k;
  int n2 = d;
  for (int q = 0; q < h.k; ++q) n2 *= chi2[q];
  const int ncol2 = d * k;
  // the forward output before normalisation: C = Si-absorbed (Q [X; 0])
  for (int i = tid; i < m * ncol2; i += kSuThreads) {
    const int row = i % m, col = i / m, s_ = col % d, b = col / d;
    double v = 0.0;
    if (row < r)
      v = side == 0 ? js[kJobU + (row + ru * s_) + (size_t)mt * b] * js[kJobS + b]
                    : js[kJobV + (s_ + dv * row) + (size_t)nt * b] * js[kJobS + b];
    Y[i] = v;
  }
  __syncthreads();
  apply_reflectors(ss, m, r, Y, ncol2, false);
  // C = Y with the inverse-sqrt environments absorbed leg by leg; every stage
  // is kept (stage 0 = Y in tensor layout) for their cotangents
  double* chain = ws + kVjChainC;
  for (int i = tid; i < n2; i += kSuThreads) {
    int row, s_, b;
    split_index(h, chi2, i, row, s_, b);
    chain[i] = Y[row + (size_t)m * (s_ + d * b)];
  }
  __syncthreads();
  double* Mt = ws + kVjM;  // a transposed chi x chi environment
  int nst = 0;             // absorbed legs
  if (a.envs) {
    int st = d;
    for (int q = 0; q < h.k; ++q) {
      if (q != h.p) {
        const int c = chi2[q];
        const double* si = ss + kSideSI + q * 64;
        for (int i = tid; i < c * c; i += kSuThreads) Mt[(i / c) + c * (i % c)] = si[i];
        __syncthreads();
        absorb_any<double>(c, chain + (size_t)nst * kSuMaxN, chain + (size_t)(nst + 1) * kSuMaxN, n2, st, Mt, tid,
                           kSuThreads);
        __syncthreads();
        ++nst;
      }
      st *= chi2[q];
    }
  }
  const double* C = chain + (size_t)nst * kSuMaxN;
  // normalisation backwards: Cbar = (Abar - A <A, Abar>) / |C|
  const double* Ab = cot_out + a.cap_off[x];
  double s2 = 0.0, dt = 0.0;
  for (int i = tid; i < n2; i += kSuThreads) {
    s2 = fma(C[i], C[i], s2);
    dt = fma(C[i], Ab[i], dt);
  }
  s2 = block_sum(s2, red);
  dt = block_sum(dt, red);
  if (tid == 0) {
    const double nc = sqrt(s2);
    s_scale = (a.normalize && nc > 0.0) ? 1.0 / nc : 1.0;
    s_dot = (a.normalize && nc > 0.0) ? dt / s2 : 0.0;  // <A, Abar> / |C| with A = C / |C|
  }
  __syncthreads();
  double* cur = ws + kVjT0;
  double* nxt = ws + kVjT1;
  for (int i = tid; i < n2; i += kSuThreads) cur[i] = (Ab[i] - C[i] * s_dot) * s_scale;
  __syncthreads();
  // inverse-sqrt environments backwards, last leg first: the cotangent of each
  // matrix (M = si^T was absorbed, so dL/dsi = gram^T), then the transposed absorb
  if (a.envs) {
    double* sib = ws + kVjSiBar;
    int st_q[kMaxDeg];
    {
      int st = d;
      for (int q = 0; q < h.k; ++q) {
        st_q[q] = st;
        st *= chi2[q];
      }
    }
    int stage = nst;
    for (int q = h.k - 1; q >= 0; --q) {
      if (q == h.p) continue;
      const int c = chi2[q];
      --stage;
      if (want_env) {
        leg_gram(cur, chain + (size_t)stage * kSuMaxN, n2, st_q[q], c, Mt);
        for (int i = tid; i < c * c; i += kSuThreads) sib[q * 64 + i] = Mt[(i / c) + c * (i % c)];
      }
      absorb_any<double>(c, cur, nxt, n2, st_q[q], ss + kSideSI + q * 64, tid, kSuThreads);
      __syncthreads();
      double* t = cur;
      cur = nxt;
      nxt = t;
    }
  }
  for (int i = tid; i < n2; i += kSuThreads) {
    int row, s_, b;
    split_index(h, chi2, i, row, s_, b);
    Y[row + (size_t)m * (s_ + d * b)] = cur[i];
  }
  __syncthreads();
  // Ybar = Q [Z; 0] + Ybar_perp
  apply_reflectors(ss, m, r, Y, ncol2, true);
  for (int i = tid; i < r * ncol2; i += kSuThreads) {
    const int t = i % r, col = i / r;
    Z[i] = Y[t + (size_t)m * col];
  }
  __syncthreads();
  for (int i = tid; i < r * ncol2; i += kSuThreads) Y[(i % r) + (size_t)m * (i / r)] = 0.0;
  __syncthreads();
  apply_reflectors(ss, m, r, Y, ncol2, false);
  // in-range cotangents of the singular vectors, and of sigma
  for (int i = tid; i < (side == 0 ? mt : nt) * k; i += kSuThreads) {
    const int row = i % (side == 0 ? mt : nt), b = i / (side == 0 ? mt : nt);
    const int t = side == 0 ? row % ru : row / dv;
    const int s_ = side == 0 ? row / ru : row % dv;
    (side == 0 ? Ub : Vb)[i] = Z[t + r * (s_ + d * b)] * js[kJobS + b];
  }
  for (int b = threadIdx.x >> 5; b < k; b += kSuWarps) {
    const int lane = tid & 31;
    double acc = 0.0;
    for (int i = lane; i < r * d; i += 32) {
      const int t = i % r, s_ = i / r;
      const double f = side == 0 ? UF[(t + ru * s_) + (size_t)mt * b] : VF[(s_ + dv * t) + (size_t)nt * b];
      acc = fma(f, Z[t + r * (s_ + d * b)], acc);
    }
    acc = warp_sum(acc);
    if (lane == 0) sb[side * kSuMaxTheta + b] = 0.5 * acc * safe_inv(js[kJobS + b]);
  }
  __syncthreads();
}

// Stage 2, one CTA per gate: the truncated-SVD adjoint in range, the gate
// transposed and the bond contraction back to Rbar of both sides, the gate's
// cotangent, and the factors H of the orthogonal terms.
__global__ void __launch_bounds__(kSuThreads, 1)
    su_vjp_core_kernel(SuArgs a, const int* post_dims, double* gate_cot, double* work) {
  const int j = blockIdx.x, tid = threadIdx.x;
  if (j >= a.njobs) return;
  VjpCtx c;
  if (!vjp_ctx(a, post_dims, work, j, c)) return;
  const int k = c.k, ce = c.ce, du = c.du, dv = c.dv, D = c.D, ru = c.ru, rv = c.rv, mt = c.mt, nt = c.nt, n = c.n;
  const double* js = c.js;
  const double* full = a.svd_full + (size_t)j * kFullStride;
  const double* UF = full + kFullU;
  const double* VF = full + kFullV;
  const double* sig = full + kFullSig;
  const double* G = a.gates + (size_t)a.gate_stride * j;
  const double* RU = c.ssd[0] + kSideR;
  const double* RV = c.ssd[1] + kSideR;
  double* wj = c.wj;
  const double* Ub = wj + kVjUb;
  const double* Vb = wj + kVjVb;
  const double* sb = wj + kVjSb;
  // ---- 3: the SVD adjoint in range
  double* UtUb = wj + kVjUtUb;
  double* VtVb = wj + kVjVtVb;
  double* J = wj + kVjJ;
  for (int i = tid; i < n * k; i += kSuThreads) {
    const int a_ = i % n, c = i / n;
    double su_ = 0.0, sv_ = 0.0;
    for (int row = 0; row < mt; ++row) su_ = fma(UF[row + (size_t)mt * a_], Ub[row + (size_t)mt * c], su_);
    for (int col = 0; col < nt; ++col) sv_ = fma(VF[col + (size_t)nt * a_], Vb[col + (size_t)nt * c], sv_);
    UtUb[i] = su_;
    VtVb[i] = sv_;
  }
  __syncthreads();
  const double smax2 = sig[0] * sig[0];
  for (int i = tid; i < n * n; i += kSuThreads) {
    const int p = i % n, q = i / n;
    double v = 0.0;
    if (p == q) {
      v = p < k ? sb[p] + sb[kSuMaxTheta + p] : 0.0;
    } else if (p < k || q < k) {
      const double den = sig[q] * sig[q] - sig[p] * sig[p];
      const double F = fabs(den) > 1e-14 * smax2 ? 1.0 / den : 0.0;
      const double au = (q < k ? UtUb[p + n * q] : 0.0) - (p < k ? UtUb[q + n * p] : 0.0);
      const double av = (q < k ? VtVb[p + n * q] : 0.0) - (p < k ? VtVb[q + n * p] : 0.0);
      v = F * (au * sig[q] + sig[p] * av);
    }
    J[i] = v;
  }
  __syncthreads();
  double* UJ = wj + kVjUJ;
  double* P1 = wj + kVjP1;
  double* P2 = wj + kVjP2;
  for (int i = tid; i < mt * n; i += kSuThreads) {
    const int row = i % mt, q = i / mt;
    double acc = 0.0;
    for (int p = 0; p < n; ++p) acc = fma(UF[row + (size_t)mt * p], J[p + n * q], acc);
    UJ[i] = acc;
  }
  for (int i = tid; i < mt * k; i += kSuThreads) {
    const int row = i % mt, c = i / mt;
    double acc = Ub[i];
    for (int p = 0; p < n; ++p) acc = fma(-UF[row + (size_t)mt * p], UtUb[p + n * c], acc);
    P1[i] = acc * safe_inv(sig[c]);
  }
  for (int i = tid; i < nt * k; i += kSuThreads) {
    const int col = i % nt, c = i / nt;
    double acc = Vb[i];
    for (int p = 0; p < n; ++p) acc = fma(-VF[col + (size_t)nt * p], VtVb[p + n * c], acc);
    P2[i] = acc * safe_inv(sig[c]);
  }
  __syncthreads();
  double* Tb = wj + kVjTb;
  for (int i = tid; i < mt * nt; i += kSuThreads) {
    const int row = i % mt, col = i / mt;
    double acc = 0.0;
    for (int q = 0; q < n; ++q) acc = fma(UJ[row + (size_t)mt * q], VF[col + (size_t)nt * q], acc);
    for (int c = 0; c < k; ++c) {
      acc = fma(P1[row + (size_t)mt * c], VF[col + (size_t)nt * c], acc);
      acc = fma(UF[row + (size_t)mt * c], P2[col + (size_t)nt * c], acc);
    }
    Tb[i] = acc;
  }
  // the theta of the forward before the gate (rows iu + ru su, columns sv + dv iv)
  double* Psi = wj + kVjPsi;
  for (int i = tid; i < mt * nt; i += kSuThreads) {
    const int row = i % mt, col = i / mt;
    const int iu = row % ru, su_ = row / ru, sv_ = col % dv, iv = col / dv;
    double acc = 0.0;
    for (int e = 0; e < ce; ++e) acc = fma(RU[iu + ru * (su_ + du * e)], RV[iv + rv * (sv_ + dv * e)], acc);
    Psi[i] = acc;
  }
  __syncthreads();

  // ---- 4: through the gate and the bond contraction
  double* Phi = wj + kVjPhi;
  for (int i = tid; i < mt * nt; i += kSuThreads) {
    const int row = i % mt, col = i / mt;
    const int iu = row % ru, su_ = row / ru, sv_ = col % dv, iv = col / dv;
    double acc = 0.0;
    for (int spv = 0; spv < dv; ++spv)
      for (int spu = 0; spu < du; ++spu)
        acc = fma(G[(spu + du * spv) + D * (su_ + du * sv_)], Tb[(iu + ru * spu) + mt * (spv + dv * iv)], acc);
    Phi[i] = acc;
  }
  if (gate_cot)
    for (int i = tid; i < D * D; i += kSuThreads) {
      const int o = i % D, in = i / D;
      const int spu = o % du, spv = o / du, su_ = in % du, sv_ = in / du;
      double acc = 0.0;
      for (int iv = 0; iv < rv; ++iv)
        for (int iu = 0; iu < ru; ++iu)
          acc = fma(Tb[(iu + ru * spu) + mt * (spv + dv * iv)], Psi[(iu + ru * su_) + mt * (sv_ + dv * iv)], acc);
      gate_cot[(size_t)j * D * D + i] = acc;
    }
  __syncthreads();
  double* Rbu = wj + kVjRb;
  double* Rbv = wj + kVjSide + kVjRb;
  for (int i = tid; i < ru * du * ce; i += kSuThreads) {
    const int iu = i % ru, su_ = (i / ru) % du, e = i / (ru * du);
    double acc = 0.0;
    for (int iv = 0; iv < rv; ++iv)
      for (int sv_ = 0; sv_ < dv; ++sv_)
        acc = fma(Phi[(iu + ru * su_) + mt * (sv_ + dv * iv)], RV[iv + rv * (sv_ + dv * e)], acc);
    Rbu[i] = acc;
  }
  for (int i = tid; i < rv * dv * ce; i += kSuThreads) {
    const int iv = i % rv, sv_ = (i / rv) % dv, e = i / (rv * dv);
    double acc = 0.0;
    for (int su_ = 0; su_ < du; ++su_)
      for (int iu = 0; iu < ru; ++iu)
        acc = fma(Phi[(iu + ru * su_) + mt * (sv_ + dv * iv)], RU[iu + ru * (su_ + du * e)], acc);
    Rbv[i] = acc;
  }
  // the orthogonal parts: M[c, s', (s, e)] = sum_t (V or U)[(s', t), c] R_other[t, (s, e)],
  // H[(s'_x, c), (s_x, e)] = sum gate M / sqrt(sigma_c)
  for (int side = 0; side < 2; ++side) {
    double* ws = wj + (size_t)side * kVjSide;
    double* M = ws + kVjM;
    const int dy = side == 0 ? dv : du;  // the other side's site dimension
    for (int i = tid; i < k * dy * dy * ce; i += kSuThreads) {
      const int c = i % k, sp = (i / k) % dy, se = i / (k * dy);  // se = s + dy e
      const int s_ = se % dy, e = se / dy;
      double acc = 0.0;
      if (side == 0)
        for (int iv = 0; iv < rv; ++iv) acc = fma(VF[(sp + dv * iv) + (size_t)nt * c], RV[iv + rv * (s_ + dv * e)], acc);
      else
        for (int iu = 0; iu < ru; ++iu) acc = fma(UF[(iu + ru * sp) + (size_t)mt * c], RU[iu + ru * (s_ + du * e)], acc);
      M[i] = acc;
    }
  }
  __syncthreads();
  for (int side = 0; side < 2; ++side) {
    double* ws = wj + (size_t)side * kVjSide;
    const double* M = ws + kVjM;
    double* H = ws + kVjH;
    const int dx = side == 0 ? du : dv, dy = side == 0 ? dv : du;
    const int rowsH = dx * k;
    for (int i = tid; i < rowsH * dx * ce; i += kSuThreads) {
      const int spx = (i % rowsH) % dx, c = (i % rowsH) / dx, col = i / rowsH, sx = col % dx, e = col / dx;
      double acc = 0.0;
      for (int sy = 0; sy < dy; ++sy)
        for (int spy = 0; spy < dy; ++spy) {
          const int o = side == 0 ? spx + du * spy : spy + du * spx;
          const int in = side == 0 ? sx + du * sy : sy + du * sx;
          acc = fma(G[o + D * in], M[c + k * (spy + dy * (sy + dy * e))], acc);
        }
      H[i] = acc * safe_inv(js[kJobS + c]);
    }
  }
  __syncthreads();

}

// Stage 3, one CTA per (gate, side): Wbar = Q [Rbar; 0] + Ybar_perp H, then the
// sqrt environments backwards, into the cotangent of the site tensor.
__global__ void __launch_bounds__(kSuThreads, 2)
    su_vjp_rebuild_kernel(SuArgs a, const int* post_dims, double* cot_in, double* work, int want_env) {
  const int j = blockIdx.x >> 1, side = blockIdx.x & 1, tid = threadIdx.x;
  if (j >= a.njobs) return;
  VjpCtx c;
  if (!vjp_ctx(a, post_dims, work, j, c)) return;
  const double* ssd[2] = {c.ssd[0], c.ssd[1]};
  const SideShape* hs = c.hs;
  const int* xs = c.xs;
  const int k = c.k, ce = c.ce;
  double* wj = c.wj;
  const SideShape& h = hs[side];
  const double* ss = ssd[side];
  double* ws = wj + (size_t)side * kVjSide;
  const double* Y = ws + kVjY;
  const double* Rb = ws + kVjRb;
  const double* H = ws + kVjH;
  double* W = ws + kVjW;
  const int x = xs[side], m = h.m, d = h.d, r = (int)ss[kSideMeta], ncol = d * ce, rowsH = d * k;
  for (int i = tid; i < m * ncol; i += kSuThreads) W[i] = (i % m) < r ? Rb[(i % m) + r * (i / m)] : 0.0;
  __syncthreads();
  apply_reflectors(ss, m, r, W, ncol, false);
  for (int i = tid; i < m * ncol; i += kSuThreads) {
    const int row = i % m, col = i / m;
    double acc = W[i];
    for (int q = 0; q < rowsH; ++q) acc = fma(Y[row + (size_t)m * q], H[q + rowsH * col], acc);
    W[i] = acc;
  }
  __syncthreads();
  double* cur = ws + kVjT0;
  double* nxt = ws + kVjT1;
  for (int i = tid; i < h.n; i += kSuThreads) {
    int row, s_, b;
    split_index(h, h.chi, i, row, s_, b);
    cur[i] = W[row + (size_t)m * (s_ + d * b)];
  }
  __syncthreads();
  if (a.envs) {
    double* Mt = ws + kVjM;
    const double* sq0 = a.side_sqrt + (size_t)(2 * j + side) * kSqrtStride;
    int st_q[kMaxDeg];
    {
      int st = d;
      for (int q = 0; q < h.k; ++q) {
        st_q[q] = st;
        st *= h.chi[q];
      }
    }
    // with the environments' cotangents wanted: the forward's stages A, A S_q0,
    // A S_q0 S_q1, ... (B = the last), recomputed from the site tensor
    double* chain = ws + kVjChainB;
    int stage = 0;
    if (want_env) {
      const double* A = a.tens + a.cap_off[x];
      for (int i = tid; i < h.n; i += kSuThreads) chain[i] = A[i];
      __syncthreads();
      for (int q = 0; q < h.k; ++q) {
        if (q == h.p) continue;
        absorb_any<double>(h.chi[q], chain + (size_t)stage * kSuMaxN, chain + (size_t)(stage + 1) * kSuMaxN, h.n,
                           st_q[q], sq0 + q * 64, tid, kSuThreads);
        __syncthreads();
        ++stage;
      }
    }
    // sqrt environments backwards, last leg first (each S_q was absorbed as is)
    for (int q = h.k - 1; q >= 0; --q) {
      if (q == h.p) continue;
      const int c = h.chi[q];
      const double* sq = sq0 + q * 64;
      if (want_env) {
        --stage;
        leg_gram(cur, chain + (size_t)stage * kSuMaxN, h.n, st_q[q], c, ws + kVjSBar + q * 64);
      }
      for (int i = tid; i < c * c; i += kSuThreads) Mt[(i / c) + c * (i % c)] = sq[i];
      __syncthreads();
      absorb_any<double>(c, cur, nxt, h.n, st_q[q], Mt, tid, kSuThreads);
      __syncthreads();
      double* t = cur;
      cur = nxt;
      nxt = t;
    }
  }
  double* dst = cot_in + a.cap_off[x];
  for (int i = tid; i < h.n; i += kSuThreads) dst[i] = cur[i];
  __syncthreads();
}

// Stage 4 (environments' cotangents wanted), one CTA per (gate, side): for
// every other leg q, the environment M of the message into the site along q
// entered as S = f(M) = V f(L) V^T (f = sqrt) and Si (f = 1/sqrt) on the kept
// eigenvalues of (M + M^T)/2 (the forward's rule; dropped ones give f = 0), so
// dL/dM = sym(V [Lf o (V^T Sbar V) + Lg o (V^T Sibar V)] V^T), with the divided
// differences Lf_ij = (f(l_i) - f(l_j)) / (l_i - l_j) (f'(l_i) on the diagonal):
// 1 / (sqrt(l_i) + sqrt(l_j)) and -1 / (sqrt(l_i l_j) (sqrt(l_i) + sqrt(l_j))) for
// two kept eigenvalues (Daleckii-Krein).  Added to env_cot (each directed
// edge's environment serves one side of one gate of a batch).
__global__ void __launch_bounds__(kSuThreads, 1)
    su_vjp_env_kernel(SuArgs a, const int* post_dims, double* work, double* env_cot) {
  const int j = blockIdx.x >> 1, side = blockIdx.x & 1, tid = threadIdx.x;
  if (j >= a.njobs || !a.envs) return;
  VjpCtx c;
  if (!vjp_ctx(a, post_dims, work, j, c)) return;
  const SideShape& h = c.hs[side];
  const int x = c.xs[side];
  double* ws = c.wj + (size_t)side * kVjSide;
  // scratch for the eigen-decomposition (the side's M region is free now)
  double* E = ws + kVjM;
  double* Sd = E;            // 64: S (recomputed)
  double* Sid = E + 64;      // 64: Si (recomputed)
  double* A8 = E + 128;      // 64
  double* V8 = E + 192;      // 64
  double* sig = E + 256;     // 64
  double* T1 = E + 320;      // 64
  double* T2 = E + 384;      // 64
  double* red = E + 448;     // 32
  double* aux = E + 480;     // 192
  double* wk = E + 672;      // 256: SVD work
  double* ex = E + 928;      // 256: SVD extra
  int* iord = reinterpret_cast<int*>(E + 1184);  // 64
  int* iperm = iord + 64;                         // 64
  __shared__ int s_flag;
  SvdBufs sb{wk, aux, aux + 64, aux + 128, iperm, iord, &s_flag, red, ex};
  for (int q = 0; q < h.k; ++q) {
    if (q == h.p) continue;
    const int cq = h.chi[q];
    const int f = a.leg_edge[a.leg_ptr[x] + q];
    const int de_in = a.edge_u[f] == x ? 2 * f + 1 : 2 * f;
    const double* env = a.envs + (size_t)de_in * a.chimax * a.chimax;
    cta_env_sqrt(env, cq, Sd, Sid, A8, V8, sig, sb);
    // the kept count, by the forward's rule
    __shared__ int s_keep;
    if (tid == 0) {
      double tot = 0.0;
      for (int i = 0; i < cq; ++i) tot += sig[i];
      if (tot == 0.0) tot = 1.0;
      int kk = cq;
      double disc = 0.0;
      while (kk > 1 && disc + sig[kk - 1] <= 10.0 * 2.220446049250313e-16 * tot) {
        disc += sig[kk - 1];
        --kk;
      }
      s_keep = kk;
    }
    __syncthreads();
    const int kk = s_keep;
    const double* sbar = ws + kVjSBar + q * 64;
    const double* sibar = ws + kVjSiBar + q * 64;
    // T1 = V^T Sbar V, T2 = V^T Sibar V
    for (int i = tid; i < cq * cq; i += kSuThreads) {
      const int p_ = i % cq, r_ = i / cq;
      double a1 = 0.0, a2 = 0.0;
      for (int u = 0; u < cq; ++u)
        for (int v = 0; v < cq; ++v) {
          const double w = V8[u + cq * p_] * V8[v + cq * r_];
          a1 = fma(w, sbar[u + cq * v], a1);
          a2 = fma(w, sibar[u + cq * v], a2);
        }
      T1[i] = a1;
      T2[i] = a2;
    }
    __syncthreads();
    // divided differences, in place: T1 <- Lf o T1 + Lg o T2
    for (int i = tid; i < cq * cq; i += kSuThreads) {
      const int p_ = i % cq, r_ = i / cq;
      const bool kp = p_ < kk, kr = r_ < kk;
      double lf = 0.0, lg = 0.0;
      if (kp && kr) {
        const double sp = sqrt(sig[p_]), sr = sqrt(sig[r_]);
        lf = 1.0 / (sp + sr);
        lg = -1.0 / (sp * sr * (sp + sr));
      } else if (kp || kr) {  // one kept, one dropped (f = 0 there)
        const double lk = kp ? sig[p_] : sig[r_], ld = kp ? sig[r_] : sig[p_];
        const double den = lk - ld;
        if (den > 0.0) {
          lf = sqrt(lk) / den;
          lg = 1.0 / (sqrt(lk) * den);
        }
      }
      T1[i] = lf * T1[i] + lg * T2[i];
    }
    __syncthreads();
    // V T1 V^T, symmetrised (the forward used (M + M^T) / 2)
    for (int i = tid; i < cq * cq; i += kSuThreads) {
      const int b = i % cq, a_ = i / cq;
      double acc = 0.0;
      for (int u = 0; u < cq; ++u)
        for (int v = 0; v < cq; ++v)
          acc = fma(V8[b + cq * u] * V8[a_ + cq * v] + V8[a_ + cq * u] * V8[b + cq * v], 0.5 * T1[u + cq * v], acc);
      env_cot[(size_t)de_in * a.chimax * a.chimax + i] += acc;
    }
    __syncthreads();
  }
}

}  // namespace
}  // namespace gbtn

// ---------------------------------------------------------------------------
// Complex tensors (ComplexF64): the same gate, one CTA per gate in one launch.
// apply.jl's simple_update_bp with complex arithmetic: Hermitian square roots
// of the environments (V f(lambda) V^H), Householder reflectors
// H = I - beta v v^H, theta without conjugation, a one-sided Jacobi SVD with
// complex rotations, the right factor sqrt(S) V^H, and the inverse-square-root
// environments absorbed conjugated on the other index, as
// tensordot(T, conj(s), axes=(leg, 0)).  Limits: site tensors (also with the
// bond at chi_max) <= 4096 elements, theta <= 32 x 32.
// ---------------------------------------------------------------------------
namespace gbtn {
namespace {

constexpr int kSuZMaxN = 4096;
constexpr int kSuZMaxTheta = 32;
constexpr int kZSide = kSuZMaxN + kMaxDeg * 64;  // zdouble per (gate, side) of global scratch

__device__ __forceinline__ zdouble zmul(zdouble a, zdouble b) {
  return zdouble(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
__device__ __forceinline__ zdouble zcmul(zdouble a, zdouble b) {  // conj(a) b
  return zdouble(a.re * b.re + a.im * b.im, a.re * b.im - a.im * b.re);
}
__device__ __forceinline__ zdouble zscale(double s, zdouble a) { return zdouble(s * a.re, s * a.im); }
__device__ __forceinline__ zdouble zsub(zdouble a, zdouble b) { return zdouble(a.re - b.re, a.im - b.im); }
__device__ __forceinline__ double zabs2(zdouble a) { return a.re * a.re + a.im * a.im; }
__device__ __forceinline__ zdouble zwarp_sum(zdouble x) { return zdouble(warp_sum(x.re), warp_sum(x.im)); }

// One-sided Jacobi SVD of X (m x n, m, n <= 32, ld m) with complex rotations:
// for the pair (i, j) with alpha = |x_i|^2, beta = |x_j|^2, gamma = x_i^H x_j
// = |gamma| e^{i phi}, zeta = (beta - alpha) / (2 |gamma|),
// t = sign(zeta) / (|zeta| + sqrt(1 + zeta^2)), c = 1 / sqrt(1 + t^2), s = c t:
//   x_i <- c x_i - s e^{-i phi} x_j,   x_j <- s e^{i phi} x_i + c x_j
// (the same on the columns of V, which starts as the identity), which makes
// the pair orthogonal.  Pairs in round-robin rounds of n/2 disjoint pairs, one
// warp per pair, one row per lane.  On return the columns of X are U S,
// sig their norms and ord the descending order.  Pairs whose squared norms are
// both at or below skip_rel * ||X||_F^2 are not rotated (as in the real
// Jacobi: for callers whose truncation discards all such columns).  Sweeps
// stop after one whose couplings were all at or below kJacobiLastSweep.
__device__ void cta_zjacobi(zdouble* X, int m, int n, zdouble* V, double* sig, int* ord, int* flag,
                            double skip_rel) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = tid; i < n * n; i += kSuThreads) V[i] = zdouble(i % n == i / n ? 1.0 : 0.0);
  double small = 0.0;
  if (skip_rel > 0.0) {  // every warp forms ||X||_F^2 itself (m <= 32 rows, one per lane)
    double f = 0.0;
    if (lane < m)
      for (int c = 0; c < n; ++c) f += zabs2(X[lane + m * c]);
    small = warp_sum(f) * skip_rel;
  }
  __syncthreads();
  const int n2 = n + (n & 1);
  for (int sweep = 0; sweep < kSvdMaxSweeps; ++sweep) {
    if (tid == 0) *flag = 0;
    __syncthreads();
    for (int r = 0; r < n2 - 1; ++r) {
      for (int k = warp; k < n2 / 2; k += kSuWarps) {
        const int a = k == 0 ? r : (r + k) % (n2 - 1);
        const int b = k == 0 ? n2 - 1 : (r - k + n2 - 1) % (n2 - 1);
        const int i = min(a, b), j = max(a, b);
        if (j >= n) continue;  // the padding column of an odd n
        const zdouble xi = lane < m ? X[lane + m * i] : zdouble(0.0);
        const zdouble xj = lane < m ? X[lane + m * j] : zdouble(0.0);
        const double al = warp_sum(zabs2(xi)), be = warp_sum(zabs2(xj));
        const zdouble ga = zwarp_sum(zcmul(xi, xj));
        const double ag = sqrt(zabs2(ga));
        if (ag > kJacobiTol * sqrt(al * be) && al > kJacobiTiny && be > kJacobiTiny && fmax(al, be) > small) {
          const double z = (be - al) / (2.0 * ag);
          const double t = (z >= 0.0 ? 1.0 : -1.0) / (fabs(z) + sqrt(1.0 + z * z));
          const double c = 1.0 / sqrt(1.0 + t * t), s = c * t;
          const zdouble se(s * ga.re / ag, s * ga.im / ag), sec(se.re, -se.im);
          if (lane < m) {
            X[lane + m * i] = zsub(zscale(c, xi), zmul(sec, xj));
            X[lane + m * j] = zmul(se, xi) + zscale(c, xj);
          }
          if (lane < n) {
            const zdouble vi = V[lane + n * i], vj = V[lane + n * j];
            V[lane + n * i] = zsub(zscale(c, vi), zmul(sec, vj));
            V[lane + n * j] = zmul(se, vi) + zscale(c, vj);
          }
          if (lane == 0) atomicOr(flag, ag * ag > kJacobiLastSweep * kJacobiLastSweep * al * be ? 3 : 1);
        }
      }
      __syncthreads();
    }
    const int rotated = *flag;
    __syncthreads();
    if ((rotated & 2) == 0) break;  // nothing rotated, or only couplings the next sweep would not see
  }
  for (int i = warp; i < n; i += kSuWarps) {
    const zdouble x = lane < m ? X[lane + m * i] : zdouble(0.0);
    const double s2 = warp_sum(zabs2(x));
    if (lane == 0) sig[i] = sqrt(s2);
  }
  __syncthreads();
  if (tid == 0) {
    for (int i = 0; i < n; ++i) ord[i] = i;
    for (int i = 1; i < n; ++i) {  // stable insertion sort, descending
      const int o = ord[i];
      int q = i;
      while (q > 0 && sig[ord[q - 1]] < sig[o]) {
        ord[q] = ord[q - 1];
        --q;
      }
      ord[q] = o;
    }
  }
  __syncthreads();
}

// sqrt and inverse sqrt of the Hermitian part of a chi x chi message
// (map_eigvals, apply.jl:9-25): eigenvalues sorted by magnitude, the tail
// whose summed magnitude is within 10 eps of the total dropped.
__device__ void cta_zenv_sqrt(const zdouble* env, int chi, zdouble* S, zdouble* Si, zdouble* A, zdouble* V,
                              double* sig, int* ord, int* flag) {
  const int tid = threadIdx.x;
  for (int i = tid; i < chi * chi; i += kSuThreads) {
    const int b = i % chi, a = i / chi;
    const zdouble x = env[b + chi * a], y = env[a + chi * b];
    A[i] = zdouble(0.5 * (x.re + y.re), 0.5 * (x.im - y.im));
  }
  __syncthreads();
  cta_zjacobi(A, chi, chi, V, sig, ord, flag, 0.0);
  __shared__ int s_keep;
  if (tid == 0) {
    double tot = 0.0;
    for (int j = 0; j < chi; ++j) tot += sig[j];
    if (tot == 0.0) tot = 1.0;
    int k = chi;
    double disc = 0.0;
    while (k > 1 && disc + sig[ord[k - 1]] <= 10.0 * 2.220446049250313e-16 * tot) {
      disc += sig[ord[k - 1]];
      --k;
    }
    s_keep = k;
  }
  __syncthreads();
  const int k = s_keep;
  for (int i = tid; i < chi * chi; i += kSuThreads) {
    const int b = i % chi, a = i / chi;
    zdouble s(0.0), si(0.0);
    for (int q = 0; q < k; ++q) {
      const int o = ord[q];
      const zdouble vv = zmul(V[b + chi * o], zdouble(V[a + chi * o].re, -V[a + chi * o].im));
      const double e = sqrt(sig[o]);
      s = s + zscale(e, vv);
      si = si + zscale(1.0 / e, vv);
    }
    S[i] = s;
    Si[i] = si;
  }
  __syncthreads();
}

// Householder QR of W (m x n, ld m), r = min(m, n) reflectors: column j of W
// becomes v_j (v_j[j] = x_j + e^{i arg x_j} |x|), beta[j] = 1 / (|x| (|x| + |x_j|))
// (0 for a zero column), R (r x n, ld r) the upper triangle, R_jj = -e^{i arg x_j} |x|.
__device__ void cta_zqr(zdouble* W, int m, int n, zdouble* R, double* beta, double* red) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int r = min(m, n);
  for (int i = tid; i < r * n; i += kSuThreads) R[i] = zdouble(0.0);
  __shared__ double s_beta;
  for (int j = 0; j < r; ++j) {
    double s2 = 0.0;
    for (int i = j + tid; i < m; i += kSuThreads) s2 += zabs2(W[i + (size_t)m * j]);
    s2 = block_sum(s2, red);
    if (tid == 0) {
      const double al = sqrt(s2);
      const zdouble x0 = W[j + (size_t)m * j];
      const double a0 = sqrt(zabs2(x0));
      if (al == 0.0) {
        s_beta = 0.0;
        R[j + r * j] = zdouble(0.0);
      } else {
        const zdouble ph = a0 > 0.0 ? zdouble(x0.re / a0, x0.im / a0) : zdouble(1.0);
        W[j + (size_t)m * j] = x0 + zscale(al, ph);
        s_beta = 1.0 / (al * (al + a0));
        R[j + r * j] = zscale(-al, ph);
      }
      beta[j] = s_beta;
    }
    __syncthreads();
    const double bj = s_beta;
    for (int c = j + 1 + warp; c < n; c += kSuWarps) {
      zdouble* y = W + (size_t)m * c;
      if (bj != 0.0) {
        const zdouble* v = W + (size_t)m * j;
        zdouble w(0.0);
        for (int i = j + lane; i < m; i += 32) w = w + zcmul(v[i], y[i]);
        w = zscale(bj, zwarp_sum(w));
        for (int i = j + lane; i < m; i += 32) y[i] = zsub(y[i], zmul(w, v[i]));
      }
      if (lane == 0) R[j + r * c] = y[j];
    }
    __syncthreads();
  }
}

// Y (m x nc, ld m) <- H_0 ... H_{r-1} Y with the reflectors of cta_zqr.
__device__ void cta_zapply_q(const zdouble* refl, const double* beta, int m, int r, zdouble* Y, int nc) {
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int jr = r - 1; jr >= 0; --jr) {
    const double bj = beta[jr];
    if (bj != 0.0) {
      const zdouble* v = refl + (size_t)jr * m;
      for (int c = warp; c < nc; c += kSuWarps) {
        zdouble* y = Y + (size_t)c * m;
        zdouble w(0.0);
        for (int i = jr + lane; i < m; i += 32) w = w + zcmul(v[i], y[i]);
        w = zscale(bj, zwarp_sum(w));
        for (int i = jr + lane; i < m; i += 32) y[i] = zsub(y[i], zmul(w, v[i]));
      }
    }
    __syncthreads();
  }
}

__device__ bool zsite_of(const SuArgs& a, const SuJob& job, int side, int& x, SideShape& h) {
  x = side ? job.v : job.u;
  side_shape(a, x, side ? job.pv : job.pu, h);
  const int ce = h.chi[h.p];
  const int r = min(h.m, h.d * ce);
  return h.n <= kSuZMaxN && h.m * h.d * a.chimax <= kSuZMaxN && h.d * ce <= 32 && r * h.d <= kSuZMaxTheta &&
         h.k <= kMaxDeg;
}

__global__ void __launch_bounds__(kSuThreads, 1) su_gate_z_kernel(SuArgs a, zdouble* zscr) {
  extern __shared__ __align__(16) double smem[];
  zdouble* B0 = reinterpret_cast<zdouble*>(smem);
  zdouble* B1 = B0 + kSuZMaxN;
  zdouble* RS[2] = {B1 + kSuZMaxN, B1 + kSuZMaxN + 1024};  // R of each side, r x (d chi)
  zdouble* EM = RS[1] + 1024;                              // 64: environment work
  zdouble* EV = EM + 64;                                   // 64
  zdouble* ES = EV + 64;                                   // 64: sqrt(env), then the rebuild's matrix
  zdouble* UU = ES + 64;                                   // 32 x 8: kept left factor
  zdouble* VV = UU + 256;                                  // 32 x 8: kept right factor
  double* sig = reinterpret_cast<double*>(VV + 256);       // 64
  double* sq = sig + 64;                                   // 64: sqrt of the kept singular values
  double* beta = sq + 64;                                  // 2 x 32
  double* red = beta + 64;                                 // 32
  int* ord = reinterpret_cast<int*>(red + 32);             // 64
  __shared__ int s_flag, s_k;
  __shared__ double s_scale;
  const int j = blockIdx.x, tid = threadIdx.x;
  if (j >= a.njobs) return;
  const SuJob job = a.jobs[j];
  int xs[2];
  SideShape hs[2];
  const bool ok0 = zsite_of(a, job, 0, xs[0], hs[0]), ok1 = zsite_of(a, job, 1, xs[1], hs[1]);
  if (!ok0 || !ok1) {
    if (tid == 0) atomicExch(a.status, 1);
    return;
  }
  zdouble* tens = reinterpret_cast<zdouble*>(a.tens);
  const zdouble* envs = reinterpret_cast<const zdouble*>(a.envs);
  zdouble* gscr = zscr + (size_t)j * 2 * kZSide;
  const int ce = hs[0].chi[hs[0].p];
  int rr[2];
  // ---- per side: sqrt environments, matricise, QR ----
  for (int side = 0; side < 2; ++side) {
    const SideShape& h = hs[side];
    const int x = xs[side];
    zdouble* refl = gscr + side * kZSide;
    zdouble* sis = refl + kSuZMaxN;
    const zdouble* src = tens + a.cap_off[x];
    for (int i = tid; i < h.n; i += kSuThreads) B0[i] = src[i];
    __syncthreads();
    zdouble* cur = B0;
    zdouble* nxt = B1;
    if (envs) {
      int st = h.d;
      for (int q = 0; q < h.k; ++q) {
        if (q != h.p) {
          const int f = a.leg_edge[a.leg_ptr[x] + q];
          const int de_in = a.edge_u[f] == x ? 2 * f + 1 : 2 * f;
          cta_zenv_sqrt(envs + (size_t)de_in * a.chimax * a.chimax, h.chi[q], ES, sis + q * 64, EM, EV, sig, ord,
                        &s_flag);
          absorb_any<zdouble>(h.chi[q], cur, nxt, h.n, st, ES, tid, kSuThreads);
          __syncthreads();
          zdouble* t = cur;
          cur = nxt;
          nxt = t;
        }
        st *= h.chi[q];
      }
    }
    for (int i = tid; i < h.n; i += kSuThreads) {
      int row, s, b;
      split_index(h, h.chi, i, row, s, b);
      nxt[row + (size_t)h.m * (s + h.d * b)] = cur[i];
    }
    __syncthreads();
    const int ncol = h.d * ce, r = min(h.m, ncol);
    cta_zqr(nxt, h.m, ncol, RS[side], beta + 32 * side, red);
    for (int i = tid; i < h.m * r; i += kSuThreads) refl[i] = nxt[i];
    rr[side] = r;
    __syncthreads();
  }
  // ---- theta = R_u R_v over the bond, then the gate ----
  const int du = hs[0].d, dv = hs[1].d, ru = rr[0], rv = rr[1];
  const int mt = ru * du, nt = dv * rv;
  const zdouble* RU = RS[0];
  const zdouble* RV = RS[1];
  for (int i = tid; i < mt * nt; i += kSuThreads) {
    const int row = i % mt, col = i / mt;
    const int iu = row % ru, su_ = row / ru, sv_ = col % dv, iv = col / dv;
    zdouble acc(0.0);
    for (int e = 0; e < ce; ++e) acc = mac(RU[iu + ru * (su_ + du * e)], RV[iv + rv * (sv_ + dv * e)], acc);
    B1[i] = acc;
  }
  __syncthreads();
  const zdouble* G = reinterpret_cast<const zdouble*>(a.gates) + (size_t)a.gate_stride * j;
  const int D = du * dv;
  const bool wide = mt < nt;
  for (int i = tid; i < mt * nt; i += kSuThreads) {
    const int row = i % mt, col = i / mt;
    const int iu = row % ru, spu = row / ru, spv = col % dv, iv = col / dv;
    zdouble acc(0.0);
    for (int sv_ = 0; sv_ < dv; ++sv_)
      for (int su_ = 0; su_ < du; ++su_)
        acc = mac(G[(spu + du * spv) + D * (su_ + du * sv_)], B1[(iu + ru * su_) + mt * (sv_ + dv * iv)], acc);
    if (wide)  // decompose theta^H (rows >= columns); its factors swap roles
      B0[col + nt * row] = zdouble(acc.re, -acc.im);
    else
      B0[i] = acc;
  }
  __syncthreads();
  const int M = wide ? nt : mt, N = wide ? mt : nt;
  cta_zjacobi(B0, M, N, B1, sig, ord, &s_flag, svd_skip_rel(a.cutoff, N));
  // theta = U S V^H: not wide, U = columns of B0 / sig, V = B1; wide (theta^H =
  // U' S V'^H), U = V' = B1 and V = U' = columns of B0 / sig
  if (tid == 0) {
    const int nsv = N;
    int n = nsv;
    double te = 0.0, scale = 0.0;
    for (int i = 0; i < nsv; ++i) scale += sig[i] * sig[i];
    if (a.maxdim > 0)
      while (n > a.maxdim) {
        te += sig[ord[n - 1]] * sig[ord[n - 1]];
        --n;
      }
    if (scale == 0.0) scale = 1.0;
    if (a.cutoff >= 0.0)
      while (n > 1 && te + sig[ord[n - 1]] * sig[ord[n - 1]] <= a.cutoff * scale) {
        te += sig[ord[n - 1]] * sig[ord[n - 1]];
        --n;
      }
    if (n < 1) n = 1;
    s_k = n;
    if (a.truncerr) a.truncerr[j] = te / scale;
    if (a.svals)
      for (int i = 0; i < a.maxdim; ++i) a.svals[(size_t)j * a.maxdim + i] = i < n ? sig[ord[i]] : 0.0;
    a.edim[job.e] = n;
  }
  __syncthreads();
  const int kk = s_k;
  for (int i = tid; i < mt * kk; i += kSuThreads) {
    const int row = i % mt, b = i / mt, o = ord[b];
    const double sg = sig[o] > 0.0 ? sig[o] : 1.0;
    UU[i] = wide ? B1[row + mt * o] : zscale(1.0 / sg, B0[row + mt * o]);
  }
  for (int i = tid; i < nt * kk; i += kSuThreads) {
    const int row = i % nt, b = i / nt, o = ord[b];
    const double sg = sig[o] > 0.0 ? sig[o] : 1.0;
    VV[i] = wide ? zscale(1.0 / sg, B0[row + nt * o]) : B1[row + nt * o];
  }
  if (tid < kk) sq[tid] = sqrt(sig[ord[tid]]);
  __syncthreads();
  // ---- rebuild each side: Q (core), layout, inverse-sqrt environments, normalise ----
  for (int side = 0; side < 2; ++side) {
    const SideShape& h = hs[side];
    const int x = xs[side];
    const zdouble* refl = gscr + side * kZSide;
    const zdouble* sis = refl + kSuZMaxN;
    int chi2[kMaxDeg];
    for (int q = 0; q < h.k; ++q) chi2[q] = h.chi[q];
    chi2[h.p] = kk;
    const int m = h.m, d = h.d, nc = d * kk, r = rr[side];
    int n2 = d;
    for (int q = 0; q < h.k; ++q) n2 *= chi2[q];
    // core: left U sqrt(S) [(t, s), b]; right (sqrt(S) V^H)^T: conj(V)[(s, t), b] sqrt(S)
    for (int i = tid; i < m * nc; i += kSuThreads) {
      const int row = i % m, col = i / m, s = col % d, b = col / d;
      zdouble v(0.0);
      if (row < r) {
        if (side == 0) {
          v = zscale(sq[b], UU[(row + ru * s) + mt * b]);
        } else {
          const zdouble w = VV[(s + dv * row) + nt * b];
          v = zscale(sq[b], zdouble(w.re, -w.im));
        }
      }
      B0[i] = v;
    }
    __syncthreads();
    cta_zapply_q(refl, beta + 32 * side, m, r, B0, nc);
    for (int i = tid; i < n2; i += kSuThreads) {
      int row, s, b;
      split_index(h, chi2, i, row, s, b);
      B1[i] = B0[row + (size_t)m * (s + d * b)];
    }
    __syncthreads();
    zdouble* cur = B1;
    zdouble* nxt = B0;
    if (envs) {
      int st = d;
      for (int q = 0; q < h.k; ++q) {
        if (q != h.p) {
          const int c = chi2[q];
          const zdouble* si = sis + q * 64;
          // out[b] = sum_a in[a] conj(Si[a, b]): the matrix conj(Si)^T
          for (int i = tid; i < c * c; i += kSuThreads) {
            const int bb = i % c, aa = i / c;
            const zdouble w = si[aa + c * bb];
            ES[i] = zdouble(w.re, -w.im);
          }
          __syncthreads();
          absorb_any<zdouble>(c, cur, nxt, n2, st, ES, tid, kSuThreads);
          __syncthreads();
          zdouble* t = cur;
          cur = nxt;
          nxt = t;
        }
        st *= chi2[q];
      }
    }
    double s2 = 0.0;
    if (a.normalize)
      for (int i = tid; i < n2; i += kSuThreads) s2 += zabs2(cur[i]);
    s2 = block_sum(s2, red);
    if (tid == 0) s_scale = (a.normalize && s2 > 0.0) ? 1.0 / sqrt(s2) : 1.0;
    __syncthreads();
    zdouble* dst = tens + a.cap_off[x];
    for (int i = tid; i < n2; i += kSuThreads) dst[i] = zscale(s_scale, cur[i]);
    __syncthreads();
  }
}

}  // namespace

size_t su_z_smem() {
  return sizeof(zdouble) * (2 * (size_t)kSuZMaxN + 2048 + 3 * 64 + 512) + sizeof(double) * (64 * 3 + 32) +
         sizeof(int) * 64;
}
constexpr size_t kSuZScratch = 2 * (size_t)kZSide;  // zdouble per gate

void su_launch_z(const SuArgs& a, zdouble* zscr, cudaStream_t s) {
  if (a.njobs == 0) return;
  const size_t sm = su_z_smem();
  GBTN_CUDA(cudaFuncSetAttribute(su_gate_z_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm));
  su_gate_z_kernel<<<a.njobs, kSuThreads, sm, s>>>(a, zscr);
  GBTN_CUDA(cudaGetLastError());
}

}  // namespace gbtn

namespace gbtn {

constexpr size_t kSuSideStride = kSideStride;
constexpr size_t kSuJobStride = kJobStride;
constexpr size_t kSuFullStride = kFullStride;
constexpr size_t kSuSqrtStride = kSqrtStride;
constexpr size_t kSuVjpStride = kVjStride;

// Shared memory of the three stages.
size_t su_qr_smem(bool envs) {
  return sizeof(double) * ((envs ? 2 : 1) * (size_t)kSuMaxN + 1024 + 64 + 32 + 64 * 4 + 192) + sizeof(int) * 128;
}
size_t su_svd_smem(int B) {
  return sizeof(double) * (6 * (size_t)B * B + 2048 + 64 + 32 + 192) + sizeof(int) * 128;
}
size_t su_rebuild_smem(bool envs) { return sizeof(double) * ((envs ? 2 : 1) * (size_t)kSuMaxN + 64 + 32); }

void su_launch(const SuArgs& a, cudaStream_t s) {
  if (a.njobs == 0) return;
  const bool envs = a.envs != nullptr;
  const size_t s1 = su_qr_smem(envs), s2 = su_svd_smem(a.bmax), s3 = su_rebuild_smem(envs);
  GBTN_CUDA(cudaFuncSetAttribute(su_qr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1));
  GBTN_CUDA(cudaFuncSetAttribute(su_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
  GBTN_CUDA(cudaFuncSetAttribute(su_rebuild_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s3));
  su_qr_kernel<<<2 * a.njobs, kSuThreads, s1, s>>>(a);
  GBTN_CUDA(cudaGetLastError());
  su_svd_kernel<<<a.njobs, kSuThreads, s2, s>>>(a);
  GBTN_CUDA(cudaGetLastError());
  su_rebuild_kernel<<<2 * a.njobs, kSuThreads, s3, s>>>(a);
  GBTN_CUDA(cudaGetLastError());
}

// The forward's QR and SVD stages with their adjoint outputs (the state is
// not written: edim must be a scratch copy of the bond dimensions), then the
// adjoint kernel.
void su_launch_fwd_stages(const SuArgs& a, cudaStream_t s) {
  if (a.njobs == 0) return;
  const bool envs = a.envs != nullptr;
  const size_t s1 = su_qr_smem(envs), s2 = su_svd_smem(a.bmax);
  GBTN_CUDA(cudaFuncSetAttribute(su_qr_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s1));
  GBTN_CUDA(cudaFuncSetAttribute(su_svd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)s2));
  su_qr_kernel<<<2 * a.njobs, kSuThreads, s1, s>>>(a);
  GBTN_CUDA(cudaGetLastError());
  su_svd_kernel<<<a.njobs, kSuThreads, s2, s>>>(a);
  GBTN_CUDA(cudaGetLastError());
}

// cot_out and cot_in may be the same buffer: stage 1 reads every gate site's
// cotangent before stage 3 (a later launch) writes any.
void su_launch_vjp_kernel(const SuArgs& a, const int* post_dims, const double* cot_out, double* cot_in,
                          double* gate_cot, double* env_cot, double* work, cudaStream_t s) {
  if (a.njobs == 0) return;
  const int want_env = env_cot && a.envs ? 1 : 0;
  su_vjp_side_kernel<<<2 * a.njobs, kSuThreads, 0, s>>>(a, post_dims, cot_out, work, want_env);
  GBTN_CUDA(cudaGetLastError());
  su_vjp_core_kernel<<<a.njobs, kSuThreads, 0, s>>>(a, post_dims, gate_cot, work);
  GBTN_CUDA(cudaGetLastError());
  su_vjp_rebuild_kernel<<<2 * a.njobs, kSuThreads, 0, s>>>(a, post_dims, cot_in, work, want_env);
  GBTN_CUDA(cudaGetLastError());
  if (want_env) {
    su_vjp_env_kernel<<<2 * a.njobs, kSuThreads, 0, s>>>(a, post_dims, work, env_cot);
    GBTN_CUDA(cudaGetLastError());
  }
}

}  // namespace gbtn

// ---------------------------------------------------------------------------
// Host side: the simple-update state and its C ABI
// ---------------------------------------------------------------------------

struct gbtn_su {
  gbtn_ctx* ctx = nullptr;
  cudaStream_t stream = nullptr;
  int nv = 0, ne = 0, chimax = 0;
  bool cplx = false;  // complex tensors: interleaved (re, im) doubles
  int es() const { return cplx ? 2 : 1; }
  std::vector<int> eu, ev, leg_ptr, leg_edge, dsite, edim;
  std::vector<long long> cap_off;
  long long cap_total = 0;
  int *d_leg_ptr = nullptr, *d_leg_edge = nullptr, *d_edge_u = nullptr, *d_dsite = nullptr, *d_edim = nullptr;
  int* d_status = nullptr;
  long long* d_cap_off = nullptr;
  double* d_tens = nullptr;
  // adjoint scratch, kept between calls and grown on demand (device), and a
  // pinned host staging buffer for cotangents
  void* d_vjp = nullptr;
  size_t vjp_bytes = 0;
  double* h_stage = nullptr;
  size_t stage_bytes = 0;
  ~gbtn_su() {
    for (void* p : {(void*)d_leg_ptr, (void*)d_leg_edge, (void*)d_edge_u, (void*)d_dsite, (void*)d_edim,
                    (void*)d_status, (void*)d_cap_off, (void*)d_tens, d_vjp})
      if (p) cudaFree(p);
    if (h_stage) cudaFreeHost(h_stage);
  }
};

namespace gbtn {
cudaStream_t ctx_stream(gbtn_ctx* c);
void set_ctx_error(gbtn_ctx* c, const char* msg);
}  // namespace gbtn

namespace {

template <typename T>
T* dev_upload(const std::vector<T>& h, cudaStream_t s) {
  T* p = nullptr;
  GBTN_CUDA(cudaMalloc(&p, std::max<size_t>(h.size(), 1) * sizeof(T)));
  if (!h.empty()) GBTN_CUDA(cudaMemcpyAsync(p, h.data(), h.size() * sizeof(T), cudaMemcpyHostToDevice, s));
  return p;
}

long long su_size(const gbtn_su* S, int v) {
  long long n = S->dsite[v];
  for (int q = S->leg_ptr[v]; q < S->leg_ptr[v + 1]; ++q) n *= S->edim[S->leg_edge[q]];
  return n;
}

void su_pull_dims(gbtn_su* S) {
  GBTN_CUDA(cudaMemcpyAsync(S->edim.data(), S->d_edim, sizeof(int) * S->ne, cudaMemcpyDeviceToHost, S->stream));
  GBTN_CUDA(cudaStreamSynchronize(S->stream));
}

int su_fail(gbtn_su* S, int code, const char* msg) {
  if (S && S->ctx) gbtn::set_ctx_error(S->ctx, msg);
  return code;
}

}  // namespace

using gbtn::SuArgs;
using gbtn::SuJob;

// The record of a taped gbtn_su_apply: per batch of vertex-disjoint gates
// the tensors and bond dimensions before it (device snapshots), the final
// state, and the gates, environments and options, for gbtn_su_tape_vjp.
struct gbtn_su_tape {
  gbtn_su* su = nullptr;
  int n_gates = 0, per_gate = 0, md = 0, normalize = 0, bmax = 0;
  long long gsz = 0;
  double cutoff = -1.0;
  double* d_gates = nullptr;
  double* d_envs = nullptr;
  SuJob* d_jobs = nullptr;
  std::vector<std::pair<int, int>> batches;
  std::vector<double*> d_tens_snap;  // before batch b; the last one after all
  std::vector<int*> d_edim_snap;
  std::vector<int> dims_before;
  ~gbtn_su_tape() {
    for (void* p : {(void*)d_gates, (void*)d_envs, (void*)d_jobs})
      if (p) cudaFree(p);
    for (double* p : d_tens_snap) cudaFree(p);
    for (int* p : d_edim_snap) cudaFree(p);
  }
};

namespace {

void tape_snapshot(gbtn_su* S, gbtn_su_tape* T, cudaStream_t s) {
  double* t = nullptr;
  int* d = nullptr;
  GBTN_CUDA(cudaMalloc(&t, sizeof(double) * std::max<long long>(S->cap_total, 1)));
  T->d_tens_snap.push_back(t);
  GBTN_CUDA(cudaMalloc(&d, sizeof(int) * std::max(S->ne, 1)));
  T->d_edim_snap.push_back(d);
  GBTN_CUDA(cudaMemcpyAsync(t, S->d_tens, sizeof(double) * S->cap_total, cudaMemcpyDeviceToDevice, s));
  if (S->ne) GBTN_CUDA(cudaMemcpyAsync(d, S->d_edim, sizeof(int) * S->ne, cudaMemcpyDeviceToDevice, s));
}

// Scratch of the adjoint for up to `chunk` gates at a time, plus the
// cotangent buffer (capacity layout), a staging copy and the gate
// cotangents, carved from the state's adjoint buffer.
struct VjpScratch {
  double *q = nullptr, *js = nullptr, *full = nullptr, *sq = nullptr, *work = nullptr;
  double *cot = nullptr, *stage = nullptr, *gc = nullptr, *env = nullptr;
  int* edim_fwd = nullptr;
  int chunk = 0;
  VjpScratch(gbtn_su* S, int max_jobs, long long gc_elems) {
    chunk = std::max(1, std::min(max_jobs, 2 * 152));
    const size_t cap = (size_t)std::max<long long>(S->cap_total, 1);
    const size_t sizes[] = {(size_t)chunk * 2 * gbtn::kSuSideStride, (size_t)chunk * gbtn::kSuJobStride,
                            (size_t)chunk * gbtn::kSuFullStride,     (size_t)chunk * 2 * gbtn::kSuSqrtStride,
                            (size_t)chunk * gbtn::kSuVjpStride,      cap,
                            cap,                                     (size_t)std::max<long long>(gc_elems, 1),
                            (size_t)std::max(2 * S->ne, 1) * S->chimax * S->chimax,
                            (size_t)std::max(S->ne, 1)};
    size_t total = 0;
    for (size_t n : sizes) total += (n + 31) / 32 * 32;
    const size_t bytes = total * sizeof(double);
    if (S->vjp_bytes < bytes) {
      if (S->d_vjp) cudaFree(S->d_vjp);
      S->d_vjp = nullptr;
      S->vjp_bytes = 0;
      GBTN_CUDA(cudaMalloc(&S->d_vjp, bytes));
      S->vjp_bytes = bytes;
    }
    double* p = static_cast<double*>(S->d_vjp);
    double** dst[] = {&q, &js, &full, &sq, &work, &cot, &stage, &gc, &env};
    for (int i = 0; i < 9; ++i) {
      *dst[i] = p;
      p += (sizes[i] + 31) / 32 * 32;
    }
    edim_fwd = reinterpret_cast<int*>(p);
  }
};

// Adjoint of one batch of vertex-disjoint gates at the state's current
// tensors and bond dimensions.  Cotangents: device, capacity layout (cot_out
// and cot_in may be the same buffer: each gate reads its sites' cotangents
// before it writes them, and no other gate touches them).
void su_vjp_batch(gbtn_su* S, const SuJob* d_jobs, int njobs, const double* d_gates, int per_gate, long long gsz,
                  const double* d_envs, int md, double cutoff, int normalize, int bmax, const int* d_post,
                  const double* d_cot_out, double* d_cot_in, double* d_gc, double* d_env_cot, VjpScratch& w) {
  cudaStream_t s = S->stream;
  for (int j0 = 0; j0 < njobs; j0 += w.chunk) {
    SuArgs a{};
    a.jobs = d_jobs + j0;
    a.njobs = std::min(w.chunk, njobs - j0);
    a.leg_ptr = S->d_leg_ptr;
    a.leg_edge = S->d_leg_edge;
    a.edge_u = S->d_edge_u;
    a.site_dim = S->d_dsite;
    a.cap_off = S->d_cap_off;
    a.tens = S->d_tens;
    a.envs = d_envs;
    a.gates = d_gates + (per_gate ? gsz * j0 : 0);
    a.gate_stride = per_gate ? gsz : 0;
    a.maxdim = md;
    a.cutoff = cutoff;
    a.normalize = normalize;
    a.chimax = S->chimax;
    a.side_scratch = w.q;
    a.job_scratch = w.js;
    a.bmax = bmax;
    a.status = S->d_status;
    a.svd_full = w.full;
    a.side_sqrt = w.sq;
    // the forward stages write the new bond dimensions into a scratch copy
    if (S->ne)
      GBTN_CUDA(cudaMemcpyAsync(w.edim_fwd, S->d_edim, sizeof(int) * S->ne, cudaMemcpyDeviceToDevice, s));
    a.edim = w.edim_fwd;
    gbtn::su_launch_fwd_stages(a, s);
    a.edim = S->d_edim;
    gbtn::su_launch_vjp_kernel(a, d_post, d_cot_out, d_cot_in, d_gc ? d_gc + gsz * j0 : nullptr, d_env_cot, w.work, s);
  }
}

int su_bmax(const gbtn_su* S) {
  int dmax = 1;
  for (int dd : S->dsite) dmax = std::max(dmax, dd);
  return std::min(64, dmax * dmax * S->chimax);
}

// Host tensors (concatenated in vertex order with bond dimensions dims) into
// a capacity-layout device buffer (host_in) or out of it (host_out), through
// the state's pinned staging buffer and one device staging copy.
void su_scatter(gbtn_su* S, const std::vector<int>& dims, const double* host_in, double* host_out, double* dev,
                double* stage) {
  cudaStream_t s = S->stream;
  const bool to_device = host_in != nullptr;
  std::vector<long long> n(S->nv);
  long long tot = 0;
  for (int v = 0; v < S->nv; ++v) {
    long long a = S->dsite[v];
    for (int q = S->leg_ptr[v]; q < S->leg_ptr[v + 1]; ++q) a *= dims[S->leg_edge[q]];
    n[v] = a;
    tot += a;
  }
  const size_t bytes = sizeof(double) * std::max<long long>(tot, 1);
  if (S->stage_bytes < bytes) {
    if (S->h_stage) cudaFreeHost(S->h_stage);
    S->h_stage = nullptr;
    S->stage_bytes = 0;
    GBTN_CUDA(cudaHostAlloc(reinterpret_cast<void**>(&S->h_stage), bytes, cudaHostAllocDefault));
    S->stage_bytes = bytes;
  }
  if (to_device) {
    std::copy(host_in, host_in + tot, S->h_stage);
    GBTN_CUDA(cudaMemcpyAsync(stage, S->h_stage, sizeof(double) * tot, cudaMemcpyHostToDevice, s));
  }
  long long off = 0;
  for (int v = 0; v < S->nv; ++v) {
    if (to_device)
      GBTN_CUDA(cudaMemcpyAsync(dev + S->cap_off[v], stage + off, sizeof(double) * n[v], cudaMemcpyDeviceToDevice, s));
    else
      GBTN_CUDA(cudaMemcpyAsync(stage + off, dev + S->cap_off[v], sizeof(double) * n[v], cudaMemcpyDeviceToDevice, s));
    off += n[v];
  }
  if (!to_device) {
    GBTN_CUDA(cudaMemcpyAsync(S->h_stage, stage, sizeof(double) * tot, cudaMemcpyDeviceToHost, s));
    GBTN_CUDA(cudaStreamSynchronize(s));
    std::copy(S->h_stage, S->h_stage + tot, host_out);
  }
  GBTN_CUDA(cudaStreamSynchronize(s));
}

}  // namespace

extern "C" {

int gbtn_su_create(gbtn_ctx* ctx, const gbtn_graph_desc* g, int32_t chi_max, gbtn_su** out) {
  if (!ctx || !g || !out) return GBTN_ERR_INVALID;
  *out = nullptr;
  try {
    auto S = std::make_unique<gbtn_su>();
    S->ctx = ctx;
    S->cplx = g->complex_values != 0;
    S->stream = gbtn::ctx_stream(ctx);
    S->nv = g->nv;
    S->ne = g->ne;
    S->chimax = chi_max;
    if (g->nv < 1 || g->ne < 0 || chi_max < 1 || chi_max > gbtn::kMaxChi)
      return su_fail(S.get(), GBTN_ERR_INVALID, "simple update: need nv >= 1 and 1 <= chi_max <= 8");
    S->eu.assign(g->edge_u, g->edge_u + g->ne);
    S->ev.assign(g->edge_v, g->edge_v + g->ne);
    S->edim.assign(g->edge_dim, g->edge_dim + g->ne);
    S->dsite.assign(g->site_dim, g->site_dim + g->nv);
    S->leg_ptr.assign(g->leg_ptr, g->leg_ptr + g->nv + 1);
    S->leg_edge.assign(g->leg_edge, g->leg_edge + S->leg_ptr[g->nv]);
    for (int e = 0; e < g->ne; ++e)
      if (S->edim[e] < 1 || S->edim[e] > chi_max || S->eu[e] == S->ev[e] || S->eu[e] < 0 || S->ev[e] < 0 ||
          S->eu[e] >= g->nv || S->ev[e] >= g->nv)
        return su_fail(S.get(), GBTN_ERR_INVALID, "simple update: bad edge or bond dimension above chi_max");
    S->cap_off.resize(g->nv);
    long long off = 0;
    for (int v = 0; v < g->nv; ++v) {
      const int k = S->leg_ptr[v + 1] - S->leg_ptr[v];
      if (k > gbtn::kMaxDeg || S->dsite[v] < 1 || S->dsite[v] > gbtn::kMaxSite)
        return su_fail(S.get(), GBTN_ERR_UNSUPPORTED, "simple update: degree above 8 or site dimension above 8");
      long long cap = S->dsite[v];
      for (int q = 0; q < k; ++q) cap *= chi_max;
      S->cap_off[v] = off;
      off += (cap + 31) / 32 * 32;
    }
    S->cap_total = off;
    S->d_leg_ptr = dev_upload(S->leg_ptr, S->stream);
    S->d_leg_edge = dev_upload(S->leg_edge, S->stream);
    S->d_edge_u = dev_upload(S->eu, S->stream);
    S->d_dsite = dev_upload(S->dsite, S->stream);
    S->d_edim = dev_upload(S->edim, S->stream);
    S->d_cap_off = dev_upload(S->cap_off, S->stream);
    std::vector<int> zero(1, 0);
    S->d_status = dev_upload(zero, S->stream);
    GBTN_CUDA(cudaMalloc(&S->d_tens, sizeof(double) * S->es() * std::max<long long>(S->cap_total, 1)));
    GBTN_CUDA(cudaMemsetAsync(S->d_tens, 0, sizeof(double) * S->es() * std::max<long long>(S->cap_total, 1),
                              S->stream));
    GBTN_CUDA(cudaStreamSynchronize(S->stream));
    *out = S.release();
    return GBTN_OK;
  } catch (const std::exception& e) {
    gbtn::set_ctx_error(ctx, e.what());
    return GBTN_ERR_CUDA;
  }
}

int gbtn_su_destroy(gbtn_su* S) {
  if (!S) return GBTN_OK;
  cudaStreamSynchronize(S->stream);
  delete S;
  return GBTN_OK;
}

int gbtn_su_edge_dims(gbtn_su* S, int32_t* dims) {
  if (!S || !dims) return GBTN_ERR_INVALID;
  try {
    su_pull_dims(S);
  } catch (const std::exception& e) {
    return su_fail(S, GBTN_ERR_CUDA, e.what());
  }
  std::copy(S->edim.begin(), S->edim.end(), dims);
  return GBTN_OK;
}

// Tensors with the current bond dimensions, concatenated in vertex order.
int gbtn_su_set_factors(gbtn_su* S, const double* ket) {
  if (!S || !ket) return GBTN_ERR_INVALID;
  try {
    su_pull_dims(S);
    long long off = 0;
    for (int v = 0; v < S->nv; ++v) {
      const long long n = su_size(S, v);
      GBTN_CUDA(cudaMemcpyAsync(S->d_tens + S->es() * S->cap_off[v], ket + S->es() * off,
                                sizeof(double) * S->es() * n, cudaMemcpyHostToDevice, S->stream));
      off += n;
    }
    GBTN_CUDA(cudaStreamSynchronize(S->stream));
  } catch (const std::exception& e) {
    return su_fail(S, GBTN_ERR_CUDA, e.what());
  }
  return GBTN_OK;
}

int gbtn_su_get_factors(gbtn_su* S, double* ket, int64_t capacity) {
  if (!S || !ket) return GBTN_ERR_INVALID;
  try {
    su_pull_dims(S);
    long long tot = 0;
    for (int v = 0; v < S->nv; ++v) tot += su_size(S, v);
    if (S->es() * tot > capacity) return su_fail(S, GBTN_ERR_INVALID, "simple update: output buffer too small");
    long long off = 0;
    for (int v = 0; v < S->nv; ++v) {
      const long long n = su_size(S, v);
      GBTN_CUDA(cudaMemcpyAsync(ket + S->es() * off, S->d_tens + S->es() * S->cap_off[v],
                                sizeof(double) * S->es() * n, cudaMemcpyDeviceToHost, S->stream));
      off += n;
    }
    GBTN_CUDA(cudaStreamSynchronize(S->stream));
  } catch (const std::exception& e) {
    return su_fail(S, GBTN_ERR_CUDA, e.what());
  }
  return GBTN_OK;
}

static int su_apply_impl(gbtn_su* S, int32_t n_gates, const int32_t* edges, const double* gates, int32_t per_gate,
                         const double* envs, int32_t maxdim, double cutoff, int32_t normalize, double* truncerr,
                         double* svals, gbtn_su_tape* tape) {
  if (!S || n_gates < 0 || (n_gates > 0 && (!edges || !gates))) return GBTN_ERR_INVALID;
  if (n_gates == 0) return tape ? GBTN_ERR_INVALID : GBTN_OK;
  try {
    cudaStream_t s = S->stream;
    int D = 0;
    std::vector<SuJob> jobs(n_gates);
    for (int j = 0; j < n_gates; ++j) {
      const int e = edges[j];
      if (e < 0 || e >= S->ne) return su_fail(S, GBTN_ERR_INVALID, "simple update: edge out of range");
      SuJob jb{e, S->eu[e], S->ev[e], -1, -1};
      for (int q = S->leg_ptr[jb.u]; q < S->leg_ptr[jb.u + 1]; ++q)
        if (S->leg_edge[q] == e) jb.pu = q - S->leg_ptr[jb.u];
      for (int q = S->leg_ptr[jb.v]; q < S->leg_ptr[jb.v + 1]; ++q)
        if (S->leg_edge[q] == e) jb.pv = q - S->leg_ptr[jb.v];
      jobs[j] = jb;
      const int dd = S->dsite[jb.u] * S->dsite[jb.v];
      if (j == 0) D = dd;
      if (per_gate && dd != D) return su_fail(S, GBTN_ERR_INVALID, "simple update: per-gate operators need equal sizes");
    }
    const long long gsz = (long long)D * D;  // elements (complex plans: interleaved pairs)
    const int es = S->es();
    double* d_gates = nullptr;
    GBTN_CUDA(cudaMalloc(&d_gates, sizeof(double) * es * gsz * (per_gate ? n_gates : 1)));
    std::unique_ptr<double, decltype(&cudaFree)> g_guard(d_gates, cudaFree);
    GBTN_CUDA(cudaMemcpyAsync(d_gates, gates, sizeof(double) * es * gsz * (per_gate ? n_gates : 1),
                              cudaMemcpyHostToDevice, s));
    double* d_envs = nullptr;
    if (envs) {
      const long long ne2 = es * 2LL * S->ne * S->chimax * S->chimax;
      GBTN_CUDA(cudaMalloc(&d_envs, sizeof(double) * std::max<long long>(ne2, 1)));
      GBTN_CUDA(cudaMemcpyAsync(d_envs, envs, sizeof(double) * ne2, cudaMemcpyHostToDevice, s));
    }
    std::unique_ptr<double, decltype(&cudaFree)> e_guard(d_envs, cudaFree);
    const int md = maxdim > 0 ? std::min(maxdim, S->chimax) : S->chimax;
    double *d_te = nullptr, *d_sv = nullptr, *d_q = nullptr;
    SuJob* d_jobs = nullptr;
    GBTN_CUDA(cudaMalloc(&d_te, sizeof(double) * n_gates));
    GBTN_CUDA(cudaMalloc(&d_sv, sizeof(double) * (size_t)n_gates * md));
    GBTN_CUDA(cudaMalloc(&d_jobs, sizeof(SuJob) * n_gates));
    std::unique_ptr<double, decltype(&cudaFree)> te_guard(d_te, cudaFree), sv_guard(d_sv, cudaFree);
    std::unique_ptr<SuJob, decltype(&cudaFree)> j_guard(d_jobs, cudaFree);
    GBTN_CUDA(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(SuJob) * n_gates, cudaMemcpyHostToDevice, s));
    // batches of consecutive, vertex-disjoint gates (they commute): sequential semantics
    std::vector<std::pair<int, int>> batches;
    std::vector<int> mark(S->nv, -1);
    int start = 0, maxb = 0;
    for (int j = 0; j < n_gates; ++j) {
      if (mark[jobs[j].u] == (int)batches.size() || mark[jobs[j].v] == (int)batches.size()) {
        batches.push_back({start, j});
        maxb = std::max(maxb, j - start);
        start = j;
      }
      mark[jobs[j].u] = mark[jobs[j].v] = (int)batches.size();
    }
    batches.push_back({start, n_gates});
    maxb = std::max(maxb, n_gates - start);
    double* d_js = nullptr;
    if (S->cplx) {  // per gate: both sides' reflectors and inverse-sqrt environments
      GBTN_CUDA(cudaMalloc(&d_q, sizeof(gbtn::zdouble) * (size_t)maxb * gbtn::kSuZScratch));
    } else {
      GBTN_CUDA(cudaMalloc(&d_q, sizeof(double) * (size_t)maxb * 2 * gbtn::kSuSideStride));
      GBTN_CUDA(cudaMalloc(&d_js, sizeof(double) * (size_t)maxb * gbtn::kSuJobStride));
    }
    std::unique_ptr<double, decltype(&cudaFree)> q_guard(d_q, cudaFree), js_guard(d_js, cudaFree);
    // theta is at most (d_u min(m_u, d_u chi)) x (d_v min(m_v, d_v chi)) <= dmax^2 chi_max
    int dmax = 1;
    for (int dd : S->dsite) dmax = std::max(dmax, dd);
    const int bmax = std::min(64, dmax * dmax * S->chimax);
    if (!S->cplx) {
      // the kernels' limits on every gate's two sites, checked here before any
      // launch so that no batch is refused half-way: each bond a gate of this
      // call may grow is taken at maxdim (the device checks the same limits)
      std::vector<int> eb(S->edim);
      for (const SuJob& jb : jobs) eb[jb.e] = std::max(eb[jb.e], md);
      for (const SuJob& jb : jobs)
        for (int side = 0; side < 2; ++side) {
          const int x = side ? jb.v : jb.u, p = side ? jb.pv : jb.pu, d = S->dsite[x], ce = eb[jb.e];
          long long m = 1;
          for (int q = S->leg_ptr[x]; q < S->leg_ptr[x + 1]; ++q)
            if (q - S->leg_ptr[x] != p) m *= eb[S->leg_edge[q]];
          const long long other = m * d, r = std::min<long long>(m, (long long)d * ce);
          if (other * std::max(md, ce) > gbtn::kSuMaxN || d * ce > 32 || r * d > bmax)
            return su_fail(S, GBTN_ERR_UNSUPPORTED,
                           "simple update: a gate exceeds the kernel limits (site tensor, also with the bond at "
                           "maxdim, > 8192 elements, or theta > 64 x 64)");
        }
    }
    GBTN_CUDA(cudaMemsetAsync(S->d_status, 0, sizeof(int), s));
    if (tape) tape->dims_before = S->edim;
    for (auto& b : batches) {
      if (tape) tape_snapshot(S, tape, s);
      SuArgs a{};
      a.jobs = d_jobs + b.first;
      a.njobs = b.second - b.first;
      a.leg_ptr = S->d_leg_ptr;
      a.leg_edge = S->d_leg_edge;
      a.edge_u = S->d_edge_u;
      a.site_dim = S->d_dsite;
      a.edim = S->d_edim;
      a.cap_off = S->d_cap_off;
      a.tens = S->d_tens;
      a.envs = d_envs;
      a.gates = d_gates + (per_gate ? es * gsz * b.first : 0);
      a.gate_stride = per_gate ? gsz : 0;  // elements
      a.maxdim = md;
      a.cutoff = cutoff;
      a.normalize = normalize;
      a.chimax = S->chimax;
      a.side_scratch = d_q;
      a.job_scratch = d_js;
      a.bmax = bmax;
      a.truncerr = d_te + b.first;
      a.svals = d_sv + (size_t)b.first * md;
      a.status = S->d_status;
      if (S->cplx)
        gbtn::su_launch_z(a, reinterpret_cast<gbtn::zdouble*>(d_q), s);
      else
        gbtn::su_launch(a, s);
    }
    if (tape) {
      tape_snapshot(S, tape, s);
      tape->su = S;
      tape->n_gates = n_gates;
      tape->per_gate = per_gate;
      tape->md = md;
      tape->cutoff = cutoff;
      tape->normalize = normalize;
      tape->bmax = bmax;
      tape->gsz = gsz;
      tape->batches = batches;
      tape->d_gates = g_guard.release();
      tape->d_envs = e_guard.release();
      tape->d_jobs = j_guard.release();
    }
    int status = 0;
    GBTN_CUDA(cudaMemcpyAsync(&status, S->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    std::vector<double> te(n_gates), sv((size_t)n_gates * md);
    GBTN_CUDA(cudaMemcpyAsync(te.data(), d_te, sizeof(double) * n_gates, cudaMemcpyDeviceToHost, s));
    GBTN_CUDA(cudaMemcpyAsync(sv.data(), d_sv, sizeof(double) * sv.size(), cudaMemcpyDeviceToHost, s));
    GBTN_CUDA(cudaStreamSynchronize(s));
    if (status)
      return su_fail(S, GBTN_ERR_UNSUPPORTED,
                     S->cplx ? "simple update: a gate exceeds the complex kernel's limits (site tensor, also with the "
                               "bond at chi_max, > 4096 elements, or theta > 32 x 32)"
                             : "simple update: a gate exceeds the kernel limits (site tensor, also with the bond at maxdim, "
                               "> 8192 elements, or theta > 64 x 64)");
    if (truncerr) std::copy(te.begin(), te.end(), truncerr);
    if (svals)
      for (int j = 0; j < n_gates; ++j)
        for (int i = 0; i < maxdim; ++i) svals[(size_t)j * maxdim + i] = i < md ? sv[(size_t)j * md + i] : 0.0;
    su_pull_dims(S);
  } catch (const std::exception& e) {
    return su_fail(S, GBTN_ERR_CUDA, e.what());
  }
  return GBTN_OK;
}

int gbtn_su_apply(gbtn_su* S, int32_t n_gates, const int32_t* edges, const double* gates, int32_t per_gate,
                  const double* envs, int32_t maxdim, double cutoff, int32_t normalize, double* truncerr,
                  double* svals) {
  const gbtn::NvtxRange nvtx_range("gbtn_su_apply");
  return su_apply_impl(S, n_gates, edges, gates, per_gate, envs, maxdim, cutoff, normalize, truncerr, svals, nullptr);
}

int gbtn_su_apply_taped(gbtn_su* S, int32_t n_gates, const int32_t* edges, const double* gates, int32_t per_gate,
                        const double* envs, int32_t maxdim, double cutoff, int32_t normalize, double* truncerr,
                        double* svals, gbtn_su_tape** tape) {
  const gbtn::NvtxRange nvtx_range("gbtn_su_apply_taped");
  if (!tape) return GBTN_ERR_INVALID;
  *tape = nullptr;
  if (S && S->cplx) return su_fail(S, GBTN_ERR_UNSUPPORTED, "simple update adjoint: real tensors only");
  gbtn_su_tape* T = nullptr;
  try {
    T = new gbtn_su_tape();
  } catch (const std::bad_alloc&) {
    return su_fail(S, GBTN_ERR_NOMEM, "host allocation failed");
  }
  const int rc = su_apply_impl(S, n_gates, edges, gates, per_gate, envs, maxdim, cutoff, normalize, truncerr, svals, T);
  if (rc != GBTN_OK) {
    if (S) cudaStreamSynchronize(S->stream);
    delete T;
    return rc;
  }
  *tape = T;
  return GBTN_OK;
}

// Valid after the state was destroyed (the tape does not use it here;
// cudaFree waits for the device).
int gbtn_su_tape_destroy(gbtn_su_tape* T) {
  delete T;
  return GBTN_OK;
}

int gbtn_su_tape_vjp(gbtn_su* S, const gbtn_su_tape* T, const double* cot_out, double* cot_in, double* gate_cot,
                     double* env_cot) {
  const gbtn::NvtxRange nvtx_range("gbtn_su_tape_vjp");
  if (!S || !T || !cot_out || !cot_in) return GBTN_ERR_INVALID;
  if (T->su != S) return su_fail(S, GBTN_ERR_INVALID, "simple update adjoint: the tape belongs to another state");
  try {
    cudaStream_t s = S->stream;
    const int nb = (int)T->batches.size();
    std::vector<int> final_dims(S->ne);
    if (S->ne)
      GBTN_CUDA(cudaMemcpyAsync(final_dims.data(), T->d_edim_snap[nb], sizeof(int) * S->ne, cudaMemcpyDeviceToHost, s));
    GBTN_CUDA(cudaStreamSynchronize(s));
    int maxb = 1;
    for (auto& b : T->batches) maxb = std::max(maxb, b.second - b.first);
    VjpScratch w(S, maxb, T->gsz * T->n_gates);
    double* d_cot = w.cot;
    double* d_gc = w.gc;
    const size_t env_elems = (size_t)2 * S->ne * S->chimax * S->chimax;
    double* d_env = env_cot && T->d_envs ? w.env : nullptr;
    if (d_env) GBTN_CUDA(cudaMemsetAsync(d_env, 0, sizeof(double) * env_elems, s));
    su_scatter(S, final_dims, cot_out, nullptr, d_cot, w.stage);
    GBTN_CUDA(cudaMemsetAsync(S->d_status, 0, sizeof(int), s));
    for (int b = nb - 1; b >= 0; --b) {
      const auto& bt = T->batches[b];
      GBTN_CUDA(cudaMemcpyAsync(S->d_tens, T->d_tens_snap[b], sizeof(double) * S->cap_total, cudaMemcpyDeviceToDevice, s));
      if (S->ne)
        GBTN_CUDA(cudaMemcpyAsync(S->d_edim, T->d_edim_snap[b], sizeof(int) * S->ne, cudaMemcpyDeviceToDevice, s));
      su_vjp_batch(S, T->d_jobs + bt.first, bt.second - bt.first, T->d_gates + (T->per_gate ? T->gsz * bt.first : 0),
                   T->per_gate, T->gsz, T->d_envs, T->md, T->cutoff, T->normalize, T->bmax, T->d_edim_snap[b + 1],
                   d_cot, d_cot, d_gc + T->gsz * bt.first, d_env, w);
    }
    // back to the state the taped apply left
    GBTN_CUDA(cudaMemcpyAsync(S->d_tens, T->d_tens_snap[nb], sizeof(double) * S->cap_total, cudaMemcpyDeviceToDevice, s));
    if (S->ne) GBTN_CUDA(cudaMemcpyAsync(S->d_edim, T->d_edim_snap[nb], sizeof(int) * S->ne, cudaMemcpyDeviceToDevice, s));
    S->edim = final_dims;
    int status = 0;
    GBTN_CUDA(cudaMemcpyAsync(&status, S->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
    GBTN_CUDA(cudaStreamSynchronize(s));
    if (status) return su_fail(S, GBTN_ERR_NUMERIC, "simple update adjoint: a recomputed gate differs from the tape");
    su_scatter(S, T->dims_before, nullptr, cot_in, d_cot, w.stage);
    if (gate_cot)
      GBTN_CUDA(cudaMemcpyAsync(gate_cot, d_gc, sizeof(double) * T->gsz * T->n_gates, cudaMemcpyDeviceToHost, s));
    if (env_cot) {
      if (d_env)
        GBTN_CUDA(cudaMemcpyAsync(env_cot, d_env, sizeof(double) * env_elems, cudaMemcpyDeviceToHost, s));
      else
        std::fill(env_cot, env_cot + env_elems, 0.0);
    }
    GBTN_CUDA(cudaStreamSynchronize(s));
  } catch (const std::exception& e) {
    return su_fail(S, GBTN_ERR_CUDA, e.what());
  }
  return GBTN_OK;
}

int gbtn_su_set_edge_dims(gbtn_su* S, const int32_t* dims) {
  if (!S || !dims) return GBTN_ERR_INVALID;
  for (int e = 0; e < S->ne; ++e)
    if (dims[e] < 1 || dims[e] > S->chimax)
      return su_fail(S, GBTN_ERR_INVALID, "simple update: bond dimension outside 1..chi_max");
  try {
    S->edim.assign(dims, dims + S->ne);
    if (S->ne)
      GBTN_CUDA(cudaMemcpyAsync(S->d_edim, S->edim.data(), sizeof(int) * S->ne, cudaMemcpyHostToDevice, S->stream));
    GBTN_CUDA(cudaStreamSynchronize(S->stream));
  } catch (const std::exception& e) {
    return su_fail(S, GBTN_ERR_CUDA, e.what());
  }
  return GBTN_OK;
}

int gbtn_su_apply_vjp(gbtn_su* S, int32_t n_gates, const int32_t* edges, const double* gates, int32_t per_gate,
                      const double* envs, int32_t maxdim, double cutoff, int32_t normalize,
                      const int32_t* post_edge_dims, const double* cot_out, double* cot_in, double* gate_cot,
                      double* env_cot) {
  const gbtn::NvtxRange nvtx_range("gbtn_su_apply_vjp");
  if (!S || n_gates < 0 || (n_gates > 0 && (!edges || !gates)) || !post_edge_dims || !cot_out || !cot_in)
    return GBTN_ERR_INVALID;
  if (S->cplx) return su_fail(S, GBTN_ERR_UNSUPPORTED, "simple update adjoint: real tensors only");
  try {
    cudaStream_t s = S->stream;
    su_pull_dims(S);
    std::vector<SuJob> jobs(n_gates);
    std::vector<int> mark(S->nv, 0), gate_edge(S->ne, 0);
    int D = 0;
    for (int j = 0; j < n_gates; ++j) {
      const int e = edges[j];
      if (e < 0 || e >= S->ne) return su_fail(S, GBTN_ERR_INVALID, "simple update: edge out of range");
      SuJob jb{e, S->eu[e], S->ev[e], -1, -1};
      if (mark[jb.u] || mark[jb.v])
        return su_fail(S, GBTN_ERR_INVALID, "simple update adjoint: the gates of one call must act on disjoint vertices");
      mark[jb.u] = mark[jb.v] = 1;
      gate_edge[e] = 1;
      for (int q = S->leg_ptr[jb.u]; q < S->leg_ptr[jb.u + 1]; ++q)
        if (S->leg_edge[q] == e) jb.pu = q - S->leg_ptr[jb.u];
      for (int q = S->leg_ptr[jb.v]; q < S->leg_ptr[jb.v + 1]; ++q)
        if (S->leg_edge[q] == e) jb.pv = q - S->leg_ptr[jb.v];
      jobs[j] = jb;
      const int dd = S->dsite[jb.u] * S->dsite[jb.v];
      if (j == 0) D = dd;
      if (dd != D) return su_fail(S, GBTN_ERR_INVALID, "simple update adjoint: gates of one call need equal sizes");
    }
    std::vector<int> post(post_edge_dims, post_edge_dims + S->ne);
    for (int e = 0; e < S->ne; ++e)
      if (gate_edge[e] ? (post[e] < 1 || post[e] > S->chimax) : post[e] != S->edim[e])
        return su_fail(S, GBTN_ERR_INVALID, "simple update adjoint: post_edge_dims do not follow the gates");
    const long long gsz = (long long)D * D;
    VjpScratch w(S, std::max<int>(n_gates, 1), gsz * n_gates);
    double* d_cot = w.cot;
    const size_t env_elems = (size_t)2 * S->ne * S->chimax * S->chimax;
    double* d_env = env_cot && envs ? w.env : nullptr;
    if (d_env) GBTN_CUDA(cudaMemsetAsync(d_env, 0, sizeof(double) * env_elems, s));
    su_scatter(S, post, cot_out, nullptr, d_cot, w.stage);  // sites without a gate keep theirs (same shapes)
    if (n_gates > 0) {
      std::vector<void*> owned;
      struct Guard {
        std::vector<void*>& v;
        ~Guard() {
          for (void* p : v) cudaFree(p);
        }
      } guard{owned};
      auto dalloc = [&](size_t bytes) {
        void* p = nullptr;
        GBTN_CUDA(cudaMalloc(&p, std::max<size_t>(bytes, 8)));
        owned.push_back(p);
        return p;
      };
      double* d_gates = (double*)dalloc(sizeof(double) * gsz * (per_gate ? n_gates : 1));
      GBTN_CUDA(cudaMemcpyAsync(d_gates, gates, sizeof(double) * gsz * (per_gate ? n_gates : 1),
                                cudaMemcpyHostToDevice, s));
      double* d_envs = nullptr;
      if (envs) {
        const long long ne2 = 2LL * S->ne * S->chimax * S->chimax;
        d_envs = (double*)dalloc(sizeof(double) * ne2);
        GBTN_CUDA(cudaMemcpyAsync(d_envs, envs, sizeof(double) * ne2, cudaMemcpyHostToDevice, s));
      }
      SuJob* d_jobs = (SuJob*)dalloc(sizeof(SuJob) * n_gates);
      GBTN_CUDA(cudaMemcpyAsync(d_jobs, jobs.data(), sizeof(SuJob) * n_gates, cudaMemcpyHostToDevice, s));
      int* d_post = (int*)dalloc(sizeof(int) * std::max(S->ne, 1));
      if (S->ne) GBTN_CUDA(cudaMemcpyAsync(d_post, post.data(), sizeof(int) * S->ne, cudaMemcpyHostToDevice, s));
      double* d_gc = w.gc;
      const int md = maxdim > 0 ? std::min(maxdim, S->chimax) : S->chimax;
      GBTN_CUDA(cudaMemsetAsync(S->d_status, 0, sizeof(int), s));
      su_vjp_batch(S, d_jobs, n_gates, d_gates, per_gate, gsz, d_envs, md, cutoff, normalize, su_bmax(S), d_post,
                   d_cot, d_cot, d_gc, d_env, w);
      int status = 0;
      GBTN_CUDA(cudaMemcpyAsync(&status, S->d_status, sizeof(int), cudaMemcpyDeviceToHost, s));
      GBTN_CUDA(cudaStreamSynchronize(s));
      if (status == 2)
        return su_fail(S, GBTN_ERR_INVALID,
                       "simple update adjoint: a gate's truncation differs from post_edge_dims (not the tensors the "
                       "gates were applied to?)");
      if (status)
        return su_fail(S, GBTN_ERR_UNSUPPORTED,
                       "simple update: a gate exceeds the kernel limits (site tensor, also with the bond at maxdim, "
                       "> 8192 elements, or theta > 64 x 64)");
      if (gate_cot)
        GBTN_CUDA(cudaMemcpyAsync(gate_cot, d_gc, sizeof(double) * gsz * n_gates, cudaMemcpyDeviceToHost, s));
    }
    if (env_cot) {
      if (d_env && n_gates > 0)
        GBTN_CUDA(cudaMemcpyAsync(env_cot, d_env, sizeof(double) * env_elems, cudaMemcpyDeviceToHost, s));
      else
        std::fill(env_cot, env_cot + env_elems, 0.0);
    }
    su_scatter(S, S->edim, nullptr, cot_in, d_cot, w.stage);
  } catch (const std::exception& e) {
    return su_fail(S, GBTN_ERR_CUDA, e.what());
  }
  return GBTN_OK;
}

}  // extern "C"
