/* CFIE Kress assembly through Chebyshev panels on the host cores (test
 * infrastructure and the timed CPU baseline only; no product code calls it).
 *
 * A C restatement, threaded with OpenMP over columns, of the reference's
 * complex-k CFIE route:
 *   Kress-split entries of one component   cfie_kress.jl:436-468 and the
 *                                          Chebyshev twin
 *                                          chebyshev_euclidian_helmholtz_cfie_kress.jl:543-666
 *   diagonal with the complex log(k^2 s^2 / 4)                   ...cfie_kress.jl:588
 *   cross-component smooth terms            cfie_kress.jl:494-503
 *   Clenshaw evaluation on uniform panels   chebyshev_core.jl:114-345,
 *                                           chebyshev_bessels.jl:574-580
 *   |k r| below the cut-off -> direct Hankel values (chebyshev_bessels.jl:1190-1207)
 * The panel coefficients are built by the Python side from SciPy's AMOS
 * values (oracle/chebyshev.py); the direct values below the cut-off come from
 * the ascending series of J0, J1, Y0, Y1 (Abramowitz and Stegun 9.1.10,
 * 9.1.11), which converge to rounding for |z| < 0.2 in a dozen terms.
 */
#include <complex.h>
#include <math.h>
#include <stddef.h>
#include <stdint.h>

typedef double complex cplx;

static const double PI_ = 3.14159265358979323846;
static const double EULER_ = 0.57721566490153286061;

/* H0 and H1 of the first kind from the ascending series (|z| small). */
static void hankel01_series(cplx z, cplx* h0, cplx* h1) {
  const cplx h = 0.5 * z, q = -h * h, lg = clog(h) + EULER_;
  cplx t0 = 1.0, t1 = h;          /* (z/2)^{2m}/(m!)^2 (-1)^m and (z/2)^{2m+1}/(m!(m+1)!) (-1)^m */
  cplx j0 = 0.0, j1 = 0.0, s0 = 0.0, s1 = 0.0;
  double hm = 0.0;                 /* harmonic number H_m */
  for (int m = 0; m < 30; ++m) {
    if (m > 0) {
      t0 *= q / ((double)m * m);
      t1 *= q / ((double)m * (m + 1));
      hm += 1.0 / m;
    }
    j0 += t0;
    j1 += t1;
    s0 += hm * t0;               /* sum_m (-1)^m H_m (z/2)^{2m}/(m!)^2 */
    s1 += (2.0 * hm + 1.0 / (m + 1)) * t1;  /* (H_m + H_{m+1}) (-1)^m (z/2)^{2m+1}/(m!(m+1)!) */
    if (cabs(t0) < 1e-18 && cabs(t1) < 1e-18) break;
  }
  const cplx y0 = (2.0 / PI_) * (lg * j0 - s0);
  const cplx y1 = -(2.0 / PI_) / z + (2.0 / PI_) * lg * j1 - (1.0 / PI_) * s1;
  *h0 = j0 + I * y0;
  *h1 = j1 + I * y1;
}

/* exported for the test of the series against SciPy */
void oracle_hankel01_small(const double* z, int64_t n, double* out) {
  for (int64_t i = 0; i < n; ++i) {
    cplx a, b;
    hankel01_series(z[2 * i] + I * z[2 * i + 1], &a, &b);
    out[4 * i + 0] = creal(a);
    out[4 * i + 1] = cimag(a);
    out[4 * i + 2] = creal(b);
    out[4 * i + 3] = cimag(b);
  }
}

typedef struct {
  int n, M;
  double lo, hi, dr, inv;
  const cplx* c; /* n x (M+1), row-major */
} plan_t;

static inline cplx plan_eval(const plan_t* p, double r) {
  long q = (long)floor((r - p->lo) * p->inv);
  if (q < 0) q = 0;
  if (q > p->n - 1) q = p->n - 1;
  const double a = p->lo + q * p->dr;
  const double b = (q == p->n - 1) ? p->hi : p->lo + (q + 1) * p->dr;
  const double t = (2.0 * r - (b + a)) / (b - a);
  const cplx* c = p->c + (size_t)q * (p->M + 1);
  cplx b1 = 0.0, b2 = 0.0;
  const double u = 2.0 * t;
  for (int m = p->M; m >= 1; --m) {
    const cplx b0 = u * b1 - b2 + c[m];
    b2 = b1;
    b1 = b0;
  }
  return t * b1 - b2 + c[0];
}

static plan_t mk(int n, int M, double lo, double hi, const double* c) {
  plan_t p;
  p.n = n;
  p.M = M;
  p.lo = lo;
  p.hi = hi;
  p.dr = (hi - lo) / n;
  p.inv = 1.0 / p.dr;
  p.c = (const cplx*)c;
  return p;
}

/* Geometry: ncomp components, offs[ncomp+1] node offsets; per node x, y, x', y',
 * x'', y'', sigma (the Kress parameter) and the weight w. rcol: the Kress
 * circulant first column of every component, concatenated like the nodes.
 * Plans: H0/H1 on [hlo, hhi] with nh panels of degree Mh, J0/J1 on [0, jhi]
 * with nj panels of degree Mj; coefficient arrays are complex128.
 * out: N x N complex128, column-major. Returns 0. */
int oracle_cfie_cheb(int ncomp, const int64_t* offs, const double* x, const double* y, const double* dx,
                     const double* dy, const double* ddx, const double* ddy, const double* sig, const double* w,
                     const double* rcol, double kre, double kim, int nh, int Mh, double hlo, double hhi,
                     const double* ch0, const double* ch1, int nj, int Mj, double jhi, const double* cj0,
                     const double* cj1, double small_cut, double* out_) {
  const int64_t N = offs[ncomp];
  const cplx k = kre + I * kim, ik = I * k;
  const plan_t H0 = mk(nh, Mh, hlo, hhi, ch0), H1 = mk(nh, Mh, hlo, hhi, ch1);
  const plan_t J0 = mk(nj, Mj, 0.0, jhi, cj0), J1 = mk(nj, Mj, 0.0, jhi, cj1);
  cplx* out = (cplx*)out_;
  const double i2pi = 1.0 / (2.0 * PI_);
  const double kabs = cabs(k);
#pragma omp parallel for schedule(dynamic, 8)
  for (int64_t j = 0; j < N; ++j) {
    int b = 0;
    while (j >= offs[b + 1]) ++b;
    const double sj = sqrt(dx[j] * dx[j] + dy[j] * dy[j]);
    for (int a = 0; a < ncomp; ++a) {
      for (int64_t i = offs[a]; i < offs[a + 1]; ++i) {
        cplx v;
        if (a == b && i == j) {
          const double si = sj;
          const double kap = i2pi * (-(dx[i] * ddy[i] - dy[i] * ddx[i])) / (dx[i] * dx[i] + dy[i] * dy[i]);
          const cplx m2d = ((0.5 * I - EULER_ / PI_) - i2pi * clog(k * k * 0.25 * si * si)) * si;
          const cplx sd = rcol[offs[a]] * (-i2pi * si) + w[i] * m2d;
          v = 1.0 - (w[i] * kap + ik * sd);
        } else {
          const double ddxij = x[i] - x[j], ddyij = y[i] - y[j];
          const double r = sqrt(ddxij * ddxij + ddyij * ddyij);
          const double inv = 1.0 / r;
          const double inner = dy[j] * ddxij - dx[j] * ddyij;
          cplx h0, h1;
          if (kabs * r < small_cut || r < hlo) {
            hankel01_series(k * r, &h0, &h1);
          } else {
            h0 = plan_eval(&H0, r);
            h1 = plan_eval(&H1, r);
          }
          if (a == b) {
            const int64_t na = offs[a + 1] - offs[a];
            int64_t d = (i - offs[a]) - (j - offs[a]);
            d %= na;
            if (d < 0) d += na;
            const double Rij = rcol[offs[a] + d];
            const double st = sin(0.5 * (sig[i] - sig[j]));
            const double lt = log(4.0 * st * st);
            const cplx j0 = plan_eval(&J0, r), j1 = plan_eval(&J1, r);
            const cplx l1 = (-k * i2pi) * inner * j1 * inv;
            const cplx l2 = (0.5 * ik) * inner * h1 * inv - l1 * lt;
            const cplx dval = Rij * l1 + w[j] * l2;
            const cplx m1 = -i2pi * j0 * sj;
            const cplx m2 = 0.5 * I * h0 * sj - m1 * lt;
            const cplx sval = Rij * m1 + w[j] * m2;
            v = -(dval + ik * sval);
          } else {
            const cplx dval = w[j] * ((0.5 * ik) * inner * h1 * inv);
            const cplx sval = w[j] * (0.5 * I * h0 * sj);
            v = -(dval + ik * sval);
          }
        }
        out[i + j * N] = v;
      }
    }
  }
  return 0;
}
