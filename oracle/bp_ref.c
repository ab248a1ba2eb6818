/*
 * bp_ref.c -- FP64 C restatement of the reference's BP message update, used
 * as the timed CPU baseline.  TEST/BENCH INFRASTRUCTURE ONLY: loaded by
 * bench.py's CPU-baseline leg and by tests, never by the product library.
 *
 * Follows ITensorNetworks.jl:
 *   updated_message (src/caches/abstractbeliefpropagationcache.jl:225-239):
 *     every message is contracted on its own from the incoming messages of
 *     the source vertex (all but the one from the target) and the ket/bra
 *     site tensors, then divided by its Frobenius norm unless it is zero;
 *   update_iteration sequential (:272-287) and parallel (:294-308, restated:
 *     every message from the pre-sweep cache), with message_diff (:32-36)
 *     summed in sequence order and the mean tested against tol (:313-329).
 * Layouts are those of include/gbtn.h (column-major tensors, site index
 * first; messages M[b, a], b = bra link).  Real tensors; bra = ket.
 * The parallel sweep runs directed edges concurrently with OpenMP.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define MAXDEG 16

typedef struct {
  long long off;
  int n, d, k;
  int chi[MAXDEG], st[MAXDEG], in_de[MAXDEG], out_de[MAXDEG];
} vinfo;

/* dst[.., b, ..] = sum_a M[b + chi*a] src[.., a, ..] along the leg with stride st */
static void absorb(const double* src, double* dst, int n, int st, int chi, const double* M) {
  const int nfib = n / chi;
  for (int f = 0; f < nfib; ++f) {
    const int lo = f % st;
    const int base = lo + (f - lo) * chi;
    for (int b = 0; b < chi; ++b) {
      double y = 0.0;
      for (int a = 0; a < chi; ++a) y += M[b + chi * a] * src[base + a * st];
      dst[base + b * st] = y;
    }
  }
}

/* out[b + chi*a] = sum_fibers bra[.., b, ..] * t[.., a, ..] */
static void close_leg(const double* t, const double* bra, int n, int st, int chi, double* out) {
  for (int i = 0; i < chi * chi; ++i) out[i] = 0.0;
  const int nfib = n / chi;
  for (int f = 0; f < nfib; ++f) {
    const int lo = f % st;
    const int base = lo + (f - lo) * chi;
    for (int a = 0; a < chi; ++a) {
      const double x = t[base + a * st];
      for (int b = 0; b < chi; ++b) out[b + chi * a] += bra[base + b * st] * x;
    }
  }
}

static void update_one(const vinfo* vi, const double* fac, const double* msgs_in, const long long* moff, int leg,
                       double* w0, double* w1, double* out) {
  const double* a = fac + vi->off;
  const double* cur = a;
  double* bufs[2] = {w0, w1};
  int which = 0;
  for (int j = 0; j < vi->k; ++j) {
    if (j == leg) continue;
    absorb(cur, bufs[which], vi->n, vi->st[j], vi->chi[j], msgs_in + moff[vi->in_de[j]]);
    cur = bufs[which];
    which ^= 1;
  }
  close_leg(cur, a, vi->n, vi->st[leg], vi->chi[leg], out);
  const int c2 = vi->chi[leg] * vi->chi[leg];
  double nrm = 0.0;
  for (int i = 0; i < c2; ++i) nrm += out[i] * out[i];
  nrm = sqrt(nrm);
  if (nrm != 0.0)
    for (int i = 0; i < c2; ++i) out[i] /= nrm;
}

static double mdiff(const double* a, const double* b, int n) {
  double d = 0, na = 0, nb = 0;
  for (int i = 0; i < n; ++i) {
    d += a[i] * b[i];
    na += a[i] * a[i];
    nb += b[i] * b[i];
  }
  return 1.0 - (d * d) / (na * nb);
}

/* Returns 0 on success.  schedule: 0 sequential (seq, seqlen), 1 parallel.
 * tol < 0: no convergence test.  iters_out / diff_out may be NULL. */
int bpref_run(int nv, int ne, const int* eu, const int* ev, const int* edim, const int* sdim, const int* leg_ptr,
              const int* leg_edge, const double* fac, double* msgs, int schedule, const int* seq, int seqlen,
              int maxiter, double tol, int nthreads, int* iters_out, double* diff_out) {
  vinfo* vi = (vinfo*)calloc((size_t)nv, sizeof(vinfo));
  long long* moff = (long long*)malloc(sizeof(long long) * (size_t)(2 * ne + 1));
  int* dchi = (int*)malloc(sizeof(int) * (size_t)(2 * ne + 1));
  int* src = (int*)malloc(sizeof(int) * (size_t)(2 * ne + 1));
  int* leg = (int*)malloc(sizeof(int) * (size_t)(2 * ne + 1));
  if (!vi || !moff || !dchi || !src || !leg) return 1;
  long long off = 0;
  for (int de = 0; de < 2 * ne; ++de) {
    dchi[de] = edim[de / 2];
    moff[de] = off;
    off += (long long)dchi[de] * dchi[de];
  }
  const long long nmsg = off;
  off = 0;
  int ncap = 1;
  for (int v = 0; v < nv; ++v) {
    vi[v].off = off;
    vi[v].d = sdim[v];
    vi[v].k = leg_ptr[v + 1] - leg_ptr[v];
    if (vi[v].k > MAXDEG) return 2;
    long long n = sdim[v];
    for (int p = 0; p < vi[v].k; ++p) {
      const int e = leg_edge[leg_ptr[v] + p];
      vi[v].chi[p] = edim[e];
      vi[v].st[p] = (int)n;
      n *= edim[e];
      const int fwd = eu[e] == v;
      vi[v].out_de[p] = fwd ? 2 * e : 2 * e + 1;
      vi[v].in_de[p] = fwd ? 2 * e + 1 : 2 * e;
      src[vi[v].out_de[p]] = v;
      leg[vi[v].out_de[p]] = p;
    }
    vi[v].n = (int)n;
    if (n > ncap) ncap = (int)n;
    off += n;
  }
  (void)ev;
  double* old = (double*)malloc(sizeof(double) * (size_t)(nmsg > 0 ? nmsg : 1));
  int nth = 1;
#ifdef _OPENMP
  nth = nthreads > 0 ? nthreads : omp_get_max_threads();
#else
  (void)nthreads;
#endif
  double* work = (double*)malloc(sizeof(double) * (size_t)ncap * 2 * nth);
  double* outs = (double*)malloc(sizeof(double) * 64 * 64 * (size_t)nth);
  int it = 0;
  double mean = NAN;
  const int ndir = 2 * ne;
  double* dd = (double*)malloc(sizeof(double) * (size_t)(ndir > 0 ? ndir : 1));
  for (it = 1; it <= maxiter; ++it) {
    double sum = 0.0;
    if (schedule == 0) {
      for (int i = 0; i < seqlen; ++i) {
        const int de = seq[i];
        const int c2 = dchi[de] * dchi[de];
        update_one(&vi[src[de]], fac, msgs, moff, leg[de], work, work + ncap, outs);
        if (tol >= 0) sum += mdiff(outs, msgs + moff[de], c2);
        memcpy(msgs + moff[de], outs, sizeof(double) * c2);
      }
      mean = sum / (double)seqlen;
    } else {
      memcpy(old, msgs, sizeof(double) * (size_t)nmsg);
#pragma omp parallel for num_threads(nth) schedule(dynamic, 4)
      for (int de = 0; de < ndir; ++de) {
        int t = 0;
#ifdef _OPENMP
        t = omp_get_thread_num();
#endif
        double* w = work + (size_t)t * 2 * ncap;
        update_one(&vi[src[de]], fac, old, moff, leg[de], w, w + ncap, msgs + moff[de]);
        dd[de] = tol >= 0 ? mdiff(msgs + moff[de], old + moff[de], dchi[de] * dchi[de]) : 0.0;
      }
      for (int e = 0; e < ne; ++e) sum += dd[2 * e];
      for (int e = 0; e < ne; ++e) sum += dd[2 * e + 1];
      mean = sum / (double)ndir;
    }
    if (tol >= 0 && mean <= tol) break;
  }
  if (it > maxiter) it = maxiter;
  if (iters_out) *iters_out = it;
  if (diff_out) *diff_out = tol >= 0 ? mean : NAN;
  free(vi); free(moff); free(dchi); free(src); free(leg); free(old); free(work); free(outs); free(dd);
  return 0;
}
