/*
 * mdft_oracle.c -- CPU restatement of Mini-MDFT's excess-functional
 * convolution hot path (test infrastructure only; see mdft_oracle.h).
 *
 * Each function names the reference lines it follows.  Paths are relative to
 * the Mini_MDFT project root.  The arithmetic order of the reference is kept
 * wherever the reference fixes it (sequential loops, left-to-right products);
 * FFTs are an own mixed-radix implementation because the reference delegates
 * them to kokkos-fft (FFTW on host, cuFFT on device), which is absent here.
 */
#include "mdft_oracle.h"

#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct {
  double re, im;
} cplx;

static inline cplx cx(double re, double im) {
  cplx z;
  z.re = re;
  z.im = im;
  return z;
}
static inline cplx cadd(cplx a, cplx b) { return cx(a.re + b.re, a.im + b.im); }
static inline cplx csub(cplx a, cplx b) { return cx(a.re - b.re, a.im - b.im); }
/* Kokkos::complex operator* (complex, complex). */
static inline cplx cmul(cplx a, cplx b) {
  return cx(a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re);
}
/* Kokkos::complex operator* (complex, real). */
static inline cplx cscale(cplx a, double s) { return cx(a.re * s, a.im * s); }
static inline cplx cconj(cplx a) { return cx(a.re, -a.im); }

#define MMAX_MAX_ROT 6 /* RotationCoeffs::m_mmax_max (MDFT_Rotation.hpp:29) */
#define ROT_L 5        /* m_mmax_max - 1 */
#define ROT_M 13       /* 2 * m_mmax_max + 1 */

static const long double kPiL = 3.141592653589793238462643383279502884L;

struct mdft_oracle {
  int nx, ny, nz;
  double lx, ly, lz;
  int mmax, mrso, ntheta, nphi, npsi, no, np;
  double *kx, *ky, *kz;
  double *thetaofntheta, *wthetaofntheta, *w;
  int *pmap, *pm, *pmup, *pmu, *pmu2;
  double *wigner, *fm;
  double rot_a[ROT_L * ROT_M * ROT_M], rot_b[ROT_L * ROT_M * ROT_M];
  double rot_c[ROT_L * ROT_M], rot_d[ROT_L * ROT_M];
  int npairs;
  int* gamma_p_map;
  int* ia_map;
  int np_new, nq;
  double dq;
  cplx* mnmunukhi_q;
  int threads;
};

/* ------------------------------------------------------------------------ */
/* Math utilities (common/MDFT_Math_Utils.hpp)                               */
/* ------------------------------------------------------------------------ */

/* gauss_legendre, MDFT_Math_Utils.hpp:25-73.  Weights sum to 1 (not 2). */
void mdfto_gauss_legendre(int n, double* x, double* w) {
  int m = (n + 1) / 2;
  for (int i = 1; i <= m; ++i) {
    double xi = cos(M_PI * (i - 0.25) / (n + 0.5));
    double deltaxi = 1.0;
    double pp = 0.0;
    int guard = 0;
    while (fabs(deltaxi) > 2.220446049250313e-16 && guard < 1000) {
      double p1 = 1.0, p2 = 0.0;
      for (int j = 1; j <= n; ++j) {
        double p3 = p2;
        p2 = p1;
        p1 = ((2 * j - 1) * xi * p2 - (j - 1) * p3) / j;
      }
      pp = n * (xi * p1 - p2) / (xi * xi - 1.0);
      deltaxi = -p1 / pp;
      xi += deltaxi;
      ++guard;
    }
    x[i - 1] = xi;
    w[i - 1] = 1.0 / ((1.0 - xi * xi) * pp * pp);
    x[n - i] = -xi;
    w[n - i] = w[i - 1];
  }
}

/* norm2, MDFT_Math_Utils.hpp:74-83 */
static double norm2_3(const double* v) {
  double s = 0;
  for (int i = 0; i < 3; ++i) s += v[i] * v[i];
  return sqrt(s);
}
/* cross_product, MDFT_Math_Utils.hpp:62-71 */
static void cross3(const double* a, const double* b, double* r) {
  r[0] = a[1] * b[2] - a[2] * b[1];
  r[1] = a[2] * b[0] - a[0] * b[2];
  r[2] = a[0] * b[1] - a[1] * b[0];
}
/* L2normalize, MDFT_Math_Utils.hpp:85-93 */
static void normalize3(double* v) {
  double n = norm2_3(v);
  for (int i = 0; i < 3; ++i) v[i] = v[i] / n;
}
/* inv_index, MDFT_Math_Utils.hpp:96-100 */
static inline int inv_index(int i, int n) { return i == 0 ? 0 : n - i; }
/* prevent_underflow (complex), MDFT_Math_Utils.hpp:102-113 */
static inline cplx prevent_underflow(cplx x, double eps) {
  if (fabs(x.re) < eps) x.re = 0.0;
  if (fabs(x.im) < eps) x.im = 0.0;
  return x;
}

/* ------------------------------------------------------------------------ */
/* Wigner small-d (common/MDFT_Wigner.hpp:20-130)                            */
/* ------------------------------------------------------------------------ */
static double factorial_tab(int k) {
  /* Exact for k <= 22, which covers every index used with mmax <= 11. */
  double f = 1.0;
  for (int i = 2; i <= k; ++i) f *= (double)i;
  return f;
}

double mdfto_wigner_small_d(int m, int mu, int mup, double theta) {
  if (abs(mu) > m || abs(mup) > m) return 0.0;
  if (m == 0) return 1.0;
  if (mu == 0 || mup == 0) {
    int mu0 = mu;
    double theta0 = theta;
    if (mu == 0) {
      mu0 = mup;
      theta0 = -theta;
    }
    double x = 1.0;
    if (mu0 < 0) {
      x = pow(-1.0, mu0);
      mu0 = -mu0;
    }
    double cc = cos(theta0);
    double pm1 = 0.0, pm = 1.0;
    for (int l = mu0 + 1; l <= m; ++l) {
      double pm2 = pm1;
      pm1 = pm;
      pm = (cc * (double)(2 * l - 1) * pm1 - (double)(l + mu0 - 1) * pm2) /
           (double)(l - mu0);
    }
    return x * pow(-1.0, mu0) *
           sqrt(factorial_tab(m - mu0) / factorial_tab(m + mu0)) *
           factorial_tab(2 * mu0) / (pow(2.0, mu0) * factorial_tab(mu0)) *
           pow(sin(theta0), mu0) * pm;
  }
  double t = 0.0;
  double cc = cos(0.5 * theta), ss = sin(0.5 * theta);
  int it0 = (0 > mu - mup) ? 0 : mu - mup;
  int it1 = (m + mu < m - mup) ? m + mu : m - mup;
  for (int it = it0; it <= it1; ++it) {
    t += pow(-1.0, it) /
         (factorial_tab(m + mu - it) * factorial_tab(m - mup - it) *
          factorial_tab(it) * factorial_tab(it - mu + mup)) *
         pow(cc, 2 * m + mu - mup - 2 * it) * pow(ss, 2 * it - mu + mup);
  }
  return sqrt(factorial_tab(m + mu) * factorial_tab(m - mu) *
              factorial_tab(m + mup) * factorial_tab(m - mup)) *
         t;
}

/* ------------------------------------------------------------------------ */
/* Rotation matrices (common/MDFT_Rotation.hpp)                              */
/* ------------------------------------------------------------------------ */

/* RotationCoeffs ctor, MDFT_Rotation.hpp:33-84 */
void mdfto_rotation_coeffs(double* a, double* b, double* c, double* d) {
  const int mm = MMAX_MAX_ROT;
  double sqrtof[2 * MMAX_MAX_ROT + 2];
  for (int i = 0; i < 2 * mm + 2; ++i) sqrtof[i] = 0.0;
  for (int i = 2; i < 14; ++i) sqrtof[i] = sqrt((double)(i - 1));
  double sqrt2 = sqrt(2.0);
  memset(a, 0, sizeof(double) * ROT_L * ROT_M * ROT_M);
  memset(b, 0, sizeof(double) * ROT_L * ROT_M * ROT_M);
  memset(c, 0, sizeof(double) * ROT_L * ROT_M);
  memset(d, 0, sizeof(double) * ROT_L * ROT_M);
  for (int l = 2; l <= mm; ++l) {
    for (int m = -l; m <= l; ++m) {
      for (int m1 = -l + 1; m1 < l; ++m1) {
        int idx = ((l - 2) * ROT_M + (m + mm)) * ROT_M + (m1 + mm);
        a[idx] = sqrtof[l + m + 1] * sqrtof[l - m + 1] /
                 (sqrtof[l + m1 + 1] * sqrtof[l - m1 + 1]);
        b[idx] = sqrtof[l + m + 1] * sqrtof[l + m] /
                 (sqrt2 * sqrtof[l + m1 + 1] * sqrtof[l - m1 + 1]);
      }
      int m1 = l;
      int idx = (l - 2) * ROT_M + (m + mm);
      c[idx] = sqrt2 * sqrtof[l + m + 1] * sqrtof[l - m + 1] /
               (sqrtof[l + m1 + 1] * sqrtof[l + m1]);
      d[idx] = sqrtof[l + m + 1] * sqrtof[l + m] /
               (sqrtof[l + m1 + 1] * sqrtof[l + m1]);
    }
  }
}

/* rotation_matrix_between_complex_spherical_harmonics_lu,
 * MDFT_Rotation.hpp:103-283.  R is complex (mmax+1, 2mmax+1, 2mmax+1). */
static void rotation_matrix(const double* q, int mmax, const double* A,
                            const double* B, const double* C, const double* D,
                            cplx* R) {
  const int mm = MMAX_MAX_ROT;
  const int n2 = 2 * mmax + 1;
#define RR(l, i, j) R[((l)*n2 + (i)) * n2 + (j)]
#define AA(l, i, j) A[((l)*ROT_M + (i)) * ROT_M + (j)]
#define BB(l, i, j) B[((l)*ROT_M + (i)) * ROT_M + (j)]
#define CC(l, i) C[(l)*ROT_M + (i)]
#define DD(l, i) D[(l)*ROT_M + (i)]
  if (mmax == 0) {
    for (int i = 0; i < (mmax + 1) * n2 * n2; ++i) R[i] = cx(1.0, 0.0);
    return;
  }
  RR(0, mmax, mmax) = cx(1.0, 0.0);
  double rmat0[3], rmat1[3], rmat2[3];
  if (q[0] == 0.0 && q[1] == 0.0 && q[2] == 0.0) {
    rmat2[0] = 0.0;
    rmat2[1] = 0.0;
    rmat2[2] = 1.0;
  } else {
    rmat2[0] = q[0];
    rmat2[1] = q[1];
    rmat2[2] = q[2];
  }
  if (rmat2[0] != 0.0 || rmat2[1] != 0.0) {
    const double ez[3] = {0, 0, 1};
    cross3(ez, rmat2, rmat1);
  } else {
    const double ex[3] = {1, 0, 0};
    cross3(rmat2, ex, rmat1);
  }
  normalize3(rmat2);
  normalize3(rmat1);
  cross3(rmat1, rmat2, rmat0);

  const double inv_sqrt2 = 1.0 / sqrt(2.0);
  RR(1, mmax - 1, mmax - 1) =
      cx((rmat1[1] + rmat0[0]) * 0.5, (rmat0[1] - rmat1[0]) * 0.5);
  RR(1, mmax - 1, mmax) = cx(rmat2[0] * inv_sqrt2, rmat2[1] * inv_sqrt2);
  RR(1, mmax - 1, mmax + 1) =
      cx((rmat1[1] - rmat0[0]) * 0.5, (-rmat0[1] - rmat1[0]) * 0.5);
  RR(1, mmax, mmax - 1) = cx(rmat0[2] * inv_sqrt2, -rmat1[2] * inv_sqrt2);
  RR(1, mmax, mmax) = cx(rmat2[2], 0.0);
  RR(1, mmax, mmax + 1) = cx(-rmat0[2] * inv_sqrt2, -rmat1[2] * inv_sqrt2);
  RR(1, mmax + 1, mmax - 1) =
      cx((rmat1[1] - rmat0[0]) * 0.5, (rmat0[1] + rmat1[0]) * 0.5);
  RR(1, mmax + 1, mmax) = cx(-rmat2[0] * inv_sqrt2, rmat2[1] * inv_sqrt2);
  RR(1, mmax + 1, mmax + 1) =
      cx((rmat1[1] + rmat0[0]) * 0.5, (rmat1[0] - rmat0[1]) * 0.5);
  if (mmax == 1) return;

  for (int l = 2; l <= mmax; ++l) {
    int l1 = l - 1;
    for (int m = -l; m <= l; ++m) {
      int m1min = m > 0 ? 1 : 0;
      for (int m1 = m1min; m1 <= l - 1; ++m1) {
        if (m == -l) {
          double bt = BB(l - 2, mm - m, mm + m1);
          cplx R0 = RR(1, mmax - 1, mmax);
          cplx R1 = RR(l1, mmax + m + 1, mmax + m1);
          double f = bt * (R0.re * R1.re - R0.im * R1.im);
          double g = bt * (R0.re * R1.im + R0.im * R1.re);
          RR(l, mmax + m, mmax + m1) = cx(f, g);
        } else if (m == l) {
          double bt = BB(l - 2, mm + m, mm + m1);
          cplx R0 = RR(1, mmax + 1, mmax);
          cplx R1 = RR(l1, mmax + m - 1, mmax + m1);
          double f = bt * (R0.re * R1.re - R0.im * R1.im);
          double g = bt * (R0.re * R1.im + R0.im * R1.re);
          RR(l, mmax + m, mmax + m1) = cx(f, g);
        } else {
          double at = AA(l - 2, mm + m, mm + m1);
          double bp = BB(l - 2, mm + m, mm + m1);
          double bn = BB(l - 2, mm - m, mm + m1);
          cplx R0 = RR(1, mmax, mmax);
          cplx R1 = RR(1, mmax + 1, mmax);
          cplx R2 = RR(1, mmax - 1, mmax);
          cplx Rm0 = RR(l1, mmax + m, mmax + m1);
          cplx Rm1 = RR(l1, mmax + m + 1, mmax + m1);
          cplx Rm2 = RR(l1, mmax + m - 1, mmax + m1);
          double f = at * (R0.re * Rm0.re) +
                     bp * (R1.re * Rm2.re - R1.im * Rm2.im) +
                     bn * (R2.re * Rm1.re - R2.im * Rm1.im);
          double g = at * (R0.re * Rm0.im) +
                     bp * (R1.re * Rm2.im + R1.im * Rm2.re) +
                     bn * (R2.re * Rm1.im + R2.im * Rm1.re);
          RR(l, mmax + m, mmax + m1) = cx(f, g);
        }
        double pw = ((m + m1) % 2 == 0) ? 1.0 : -1.0;
        cplx v = RR(l, mmax + m, mmax + m1);
        RR(l, mmax - m, mmax - m1) = cx(pw * v.re, -pw * v.im);
      }
      int m1 = l;
      {
        if (m == -l) {
          double dt = DD(l - 2, mm - m);
          cplx R0 = RR(1, mmax - 1, mmax + 1);
          cplx R1 = RR(l1, mmax + m + 1, mmax + m1 - 1);
          double f = dt * (R0.re * R1.re - R0.im * R1.im);
          double g = dt * (R0.re * R1.im + R0.im * R1.re);
          RR(l, mmax + m, mmax + m1) = cx(f, g);
        } else if (m == l) {
          double dt = DD(l - 2, mm + m);
          cplx R0 = RR(1, mmax + 1, mmax + 1);
          cplx R1 = RR(l1, mmax + m - 1, mmax + m1 - 1);
          double f = dt * (R0.re * R1.re - R0.im * R1.im);
          double g = dt * (R0.re * R1.im + R0.im * R1.re);
          RR(l, mmax + m, mmax + m1) = cx(f, g);
        } else {
          double ct = CC(l - 2, mm + m);
          double dp = DD(l - 2, mm + m);
          double dn = DD(l - 2, mm - m);
          cplx R0 = RR(1, mmax, mmax + 1);
          cplx R1 = RR(1, mmax + 1, mmax + 1);
          cplx R2 = RR(1, mmax - 1, mmax + 1);
          cplx Rm0 = RR(l1, mmax + m, mmax + m1 - 1);
          cplx Rm1 = RR(l1, mmax + m + 1, mmax + m1 - 1);
          cplx Rm2 = RR(l1, mmax + m - 1, mmax + m1 - 1);
          double f = ct * (R0.re * Rm0.re - R0.im * Rm0.im) +
                     dp * (R1.re * Rm2.re - R1.im * Rm2.im) +
                     dn * (R2.re * Rm1.re - R2.im * Rm1.im);
          double g = ct * (R0.re * Rm0.im + R0.im * Rm0.re) +
                     dp * (R1.re * Rm2.im + R1.im * Rm2.re) +
                     dn * (R2.re * Rm1.im + R2.im * Rm1.re);
          RR(l, mmax + m, mmax + m1) = cx(f, g);
        }
        double pw = ((m + m1) % 2 == 0) ? 1.0 : -1.0;
        cplx v = RR(l, mmax + m, mmax + m1);
        RR(l, mmax - m, mmax - m1) = cx(pw * v.re, -pw * v.im);
      }
    }
  }
#undef RR
#undef AA
#undef BB
#undef CC
#undef DD
}

void mdfto_rotation_matrix(const double* q, int mmax, double* R) {
  double a[ROT_L * ROT_M * ROT_M], b[ROT_L * ROT_M * ROT_M];
  double c[ROT_L * ROT_M], d[ROT_L * ROT_M];
  mdfto_rotation_coeffs(a, b, c, d);
  rotation_matrix(q, mmax, a, b, c, d, (cplx*)R);
}

/* ------------------------------------------------------------------------ */
/* Mixed-radix FFT (own; the reference calls kokkos-fft)                     */
/* ------------------------------------------------------------------------ */
typedef struct {
  int n;
  cplx* tw; /* exp(-2 pi i t / n), t = 0..n-1 */
} fftplan;

static void fftplan_init(fftplan* p, int n) {
  p->n = n;
  p->tw = (cplx*)malloc(sizeof(cplx) * (size_t)(n > 0 ? n : 1));
  for (int t = 0; t < n; ++t) {
    long double ang = 2.0L * kPiL * (long double)t / (long double)n;
    p->tw[t] = cx((double)cosl(ang), -(double)sinl(ang));
  }
}
static void fftplan_free(fftplan* p) { free(p->tw); }

static int pick_radix(int n) {
  if (n % 4 == 0 && n != 8) return 4;
  if (n % 2 == 0) return 2;
  for (int r = 3; r * r <= n; r += 2)
    if (n % r == 0) return r;
  return n;
}

/* out[k] = sum_j in[j*is] * exp(sign 2 pi i j k / n); step = n0 / n. */
static void fft_rec(const cplx* in, long is, cplx* out, int n, int step,
                    const fftplan* P, int sign, cplx* work) {
  if (n == 1) {
    out[0] = in[0];
    return;
  }
  int r = pick_radix(n);
  int m = n / r;
  for (int j = 0; j < r; ++j)
    fft_rec(in + j * is, is * r, out + j * m, m, step * r, P, sign, work);
  const cplx* tw = P->tw;
  const int n0 = P->n;
  for (int k = 0; k < m; ++k) {
    cplx* v = work;
    for (int j = 0; j < r; ++j) {
      cplx t = tw[(long)j * k * step];
      if (sign > 0) t = cconj(t);
      v[j] = (j == 0 || k == 0) ? out[j * m + k] : cmul(out[j * m + k], t);
    }
    if (r == 2) {
      out[k] = cadd(v[0], v[1]);
      out[k + m] = csub(v[0], v[1]);
    } else if (r == 4) {
      cplx a0 = cadd(v[0], v[2]), a1 = csub(v[0], v[2]);
      cplx b0 = cadd(v[1], v[3]), b1 = csub(v[1], v[3]);
      /* forward: multiply b1 by -i; backward by +i */
      cplx jb1 = (sign < 0) ? cx(b1.im, -b1.re) : cx(-b1.im, b1.re);
      out[k] = cadd(a0, b0);
      out[k + m] = cadd(a1, jb1);
      out[k + 2 * m] = csub(a0, b0);
      out[k + 3 * m] = csub(a1, jb1);
    } else {
      cplx* res = work + r;
      int wstep = n0 / r;
      for (int s = 0; s < r; ++s) {
        cplx acc = v[0];
        for (int j = 1; j < r; ++j) {
          cplx t = tw[(long)((j * s) % r) * wstep];
          if (sign > 0) t = cconj(t);
          acc = cadd(acc, cmul(v[j], t));
        }
        res[s] = acc;
      }
      for (int s = 0; s < r; ++s) out[k + s * m] = res[s];
    }
  }
}

/* One pencil pass over axis `ax` of (batch, n0, n1, n2). */
static void fft_axis(cplx* data, int batch, int n0, int n1, int n2, int ax,
                     int sign) {
  int dims[3] = {n0, n1, n2};
  long strides[3] = {(long)n1 * n2, n2, 1};
  int n = dims[ax];
  if (n == 1) return;
  long stride = strides[ax];
  long total = (long)batch * n0 * n1 * n2;
  long npencil = total / n;
  fftplan P;
  fftplan_init(&P, n);
#pragma omp parallel
  {
    cplx* a = (cplx*)malloc(sizeof(cplx) * n);
    cplx* b = (cplx*)malloc(sizeof(cplx) * n);
    cplx* work = (cplx*)malloc(sizeof(cplx) * 2 * (n + 2));
#pragma omp for schedule(static)
    for (long pc = 0; pc < npencil; ++pc) {
      /* pencil pc -> base offset: decompose over the other axes */
      long base;
      if (ax == 2) {
        base = pc * n;
      } else if (ax == 1) {
        long bb = pc / n2, z = pc % n2; /* bb = batch*n0 index */
        base = bb * (long)n1 * n2 + z;
      } else {
        long bb = pc / ((long)n1 * n2), yz = pc % ((long)n1 * n2);
        base = bb * (long)n0 * n1 * n2 + yz;
      }
      for (int j = 0; j < n; ++j) a[j] = data[base + j * stride];
      fft_rec(a, 1, b, n, 1, &P, sign, work);
      for (int j = 0; j < n; ++j) data[base + j * stride] = b[j];
    }
    free(a);
    free(b);
    free(work);
  }
  fftplan_free(&P);
}

void mdfto_fft3d(double* data, int batch, int nx, int ny, int nz, int sign) {
  cplx* d = (cplx*)data;
  fft_axis(d, batch, nx, ny, nz, 2, sign);
  fft_axis(d, batch, nx, ny, nz, 1, sign);
  fft_axis(d, batch, nx, ny, nz, 0, sign);
}

/* ------------------------------------------------------------------------ */
/* Grids and orientation/projection map                                      */
/* ------------------------------------------------------------------------ */

/* SpatialGrid::kproj, MDFT_Grid.hpp:87-103 */
static void kproj(double* k, int n, double d) {
  int N1 = n / 2 + 1, N2 = (n - 1) / 2;
  for (int i = 0; i < N1; i++) k[i] = (double)i * d;
  for (int i = 0; i < N2; i++) k[i + N1] = (double)(i - N2) * d;
}

mdft_oracle* mdfto_create(int nx, int ny, int nz, double lx, double ly,
                          double lz, int mmax, int mrso) {
  if (nx <= 0 || ny <= 0 || nz <= 0 || lx <= 0 || ly <= 0 || lz <= 0 ||
      mmax <= 0 || mrso <= 0 || mmax > 11)
    return NULL;
  mdft_oracle* o = (mdft_oracle*)calloc(1, sizeof(mdft_oracle));
  o->nx = nx;
  o->ny = ny;
  o->nz = nz;
  o->lx = lx;
  o->ly = ly;
  o->lz = lz;
  o->mmax = mmax;
  o->mrso = mrso;
  o->threads = 0;
  o->kx = (double*)malloc(sizeof(double) * nx);
  o->ky = (double*)malloc(sizeof(double) * ny);
  o->kz = (double*)malloc(sizeof(double) * nz);
  kproj(o->kx, nx, 2.0 * M_PI / lx);
  kproj(o->ky, ny, 2.0 * M_PI / ly);
  kproj(o->kz, nz, 2.0 * M_PI / lz);

  /* AngularGrid, MDFT_Grid.hpp:264-398 */
  o->ntheta = mmax + 1;
  o->nphi = 2 * mmax + 1;
  o->npsi = 2 * (mmax / mrso) + 1;
  o->no = o->ntheta * o->nphi * o->npsi;
  int np = 0;
  for (int m = 0; m <= mmax; ++m)
    for (int mup = -m; mup <= m; ++mup)
      for (int mu = 0; mu <= m / mrso; ++mu) np++;
  o->np = np;
  o->thetaofntheta = (double*)malloc(sizeof(double) * o->ntheta);
  o->wthetaofntheta = (double*)malloc(sizeof(double) * o->ntheta);
  mdfto_gauss_legendre(o->ntheta, o->thetaofntheta, o->wthetaofntheta);
  for (int i = 0; i < o->ntheta; ++i) o->thetaofntheta[i] = acos(o->thetaofntheta[i]);
  o->w = (double*)malloc(sizeof(double) * o->no);
  {
    double wphi = 1.0 / (double)o->nphi;
    double wpsi = 1.0 / (double)(o->npsi * mrso);
    double qn = 8.0 * M_PI * M_PI;
    int io = 0;
    for (int it = 0; it < o->ntheta; it++)
      for (int iphi = 0; iphi < o->nphi; iphi++)
        for (int ipsi = 0; ipsi < o->npsi; ipsi++) {
          o->w[io] = o->wthetaofntheta[it] * wphi * wpsi * qn;
          io++;
        }
  }

  /* OrientationProjectionMap, MDFT_OrientationProjectionTransform.hpp:55-148 */
  int K = mmax / mrso;
  o->pmap = (int*)calloc((size_t)(mmax + 1) * (2 * mmax + 1) * (K + 1), sizeof(int));
  o->pm = (int*)malloc(sizeof(int) * np);
  o->pmup = (int*)malloc(sizeof(int) * np);
  o->pmu = (int*)malloc(sizeof(int) * np);
  o->pmu2 = (int*)malloc(sizeof(int) * np);
  int ip = 0;
  for (int m = 0; m <= mmax; ++m)
    for (int mup = -m; mup <= m; ++mup)
      for (int mu = 0; mu <= m; mu += mrso) {
        o->pmap[(m * (2 * mmax + 1) + (mup + mmax)) * (K + 1) + mu / mrso] = ip;
        o->pm[ip] = m;
        o->pmup[ip] = mup;
        o->pmu[ip] = mu;
        o->pmu2[ip] = mu / mrso;
        ip++;
      }
  o->wigner = (double*)malloc(sizeof(double) * o->ntheta * np);
  for (int p = 0; p < np; p++)
    for (int it = 0; it < o->ntheta; it++)
      o->wigner[it * np + p] =
          mdfto_wigner_small_d(o->pm[p], o->pmup[p], o->pmu[p], o->thetaofntheta[it]);
  /* OrientationProjectionTransform ctor, :233-236 */
  o->fm = (double*)malloc(sizeof(double) * (mmax + 1));
  for (int m = 0; m <= mmax; ++m) o->fm[m] = sqrt(2.0 * (double)m + 1.0);

  mdfto_rotation_coeffs(o->rot_a, o->rot_b, o->rot_c, o->rot_d);

  /* gamma_p_map, MDFT_Convolution.hpp:129-176 */
  {
    unsigned char* isok = (unsigned char*)calloc((size_t)nx * ny * nz, 1);
    int len = 0;
    for (int pass = 0; pass < 2; ++pass) {
      memset(isok, 0, (size_t)nx * ny * nz);
      len = 0;
      for (int iz = 0; iz < nz / 2 + 1; ++iz) {
        int izm = inv_index(iz, nz);
        for (int iy = 0; iy < ny; ++iy) {
          int iym = inv_index(iy, ny);
          for (int ix = 0; ix < nx; ++ix) {
            int ixm = inv_index(ix, nx);
            size_t a = ((size_t)ix * ny + iy) * nz + iz;
            size_t b = ((size_t)ixm * ny + iym) * nz + izm;
            if (isok[a] && isok[b]) continue;
            if (pass == 1) {
              o->gamma_p_map[3 * len + 0] = ix;
              o->gamma_p_map[3 * len + 1] = iy;
              o->gamma_p_map[3 * len + 2] = iz;
            }
            isok[a] = 1;
            isok[b] = 1;
            len++;
          }
        }
      }
      if (pass == 0) {
        o->npairs = len;
        o->gamma_p_map = (int*)malloc(sizeof(int) * 3 * (size_t)len);
      }
    }
    free(isok);
  }
  /* ia_map, MDFT_Convolution.hpp:178-196 */
  {
    int n2 = 2 * mmax / mrso + 1;
    o->ia_map = (int*)calloc((size_t)np * (mmax + 1) * n2, sizeof(int));
    int ia = 0;
    for (int p = 0; p < np; p++) {
      int ikhi = o->pmup[p];
      for (int in = abs(ikhi); in <= mmax; in++)
        for (int inu2 = -in / mrso; inu2 <= in / mrso; inu2++) {
          o->ia_map[(p * (mmax + 1) + in) * n2 + inu2 + mmax / mrso] = ia;
          ia++;
        }
    }
    o->np_new = ia;
  }
  return o;
}

void mdfto_destroy(mdft_oracle* o) {
  if (!o) return;
  free(o->kx);
  free(o->ky);
  free(o->kz);
  free(o->thetaofntheta);
  free(o->wthetaofntheta);
  free(o->w);
  free(o->pmap);
  free(o->pm);
  free(o->pmup);
  free(o->pmu);
  free(o->pmu2);
  free(o->wigner);
  free(o->fm);
  free(o->gamma_p_map);
  free(o->ia_map);
  free(o->mnmunukhi_q);
  free(o);
}

void mdfto_set_threads(mdft_oracle* o, int nthreads) {
  o->threads = nthreads;
#ifdef _OPENMP
  if (nthreads > 0) omp_set_num_threads(nthreads);
#endif
}

void mdfto_info(const mdft_oracle* o, int* v) {
  v[0] = o->nx;
  v[1] = o->ny;
  v[2] = o->nz;
  v[3] = o->mmax;
  v[4] = o->mrso;
  v[5] = o->ntheta;
  v[6] = o->nphi;
  v[7] = o->npsi;
  v[8] = o->no;
  v[9] = o->np;
  v[10] = o->npairs;
  v[11] = o->np_new;
  v[12] = o->nq;
}

void mdfto_kvectors(const mdft_oracle* o, double* kx, double* ky, double* kz) {
  memcpy(kx, o->kx, sizeof(double) * o->nx);
  memcpy(ky, o->ky, sizeof(double) * o->ny);
  memcpy(kz, o->kz, sizeof(double) * o->nz);
}

void mdfto_angular(const mdft_oracle* o, double* th, double* wth, double* w) {
  memcpy(th, o->thetaofntheta, sizeof(double) * o->ntheta);
  memcpy(wth, o->wthetaofntheta, sizeof(double) * o->ntheta);
  memcpy(w, o->w, sizeof(double) * o->no);
}

void mdfto_opmap(const mdft_oracle* o, int* p, int* m, int* mup, int* mu,
                 int* mu2, double* wigner) {
  int K = o->mmax / o->mrso;
  memcpy(p, o->pmap, sizeof(int) * (o->mmax + 1) * (2 * o->mmax + 1) * (K + 1));
  memcpy(m, o->pm, sizeof(int) * o->np);
  memcpy(mup, o->pmup, sizeof(int) * o->np);
  memcpy(mu, o->pmu, sizeof(int) * o->np);
  memcpy(mu2, o->pmu2, sizeof(int) * o->np);
  memcpy(wigner, o->wigner, sizeof(double) * o->ntheta * o->np);
}

/* q_max needed by the grid, MDFT_Convolution.hpp:214-231 */
double mdfto_qmax(const mdft_oracle* o) {
  double kxm = o->kx[0], kym = o->ky[0], kzm = o->kz[0];
  for (int i = 0; i < o->nx; ++i) kxm = o->kx[i] > kxm ? o->kx[i] : kxm;
  for (int i = 0; i < o->ny; ++i) kym = o->ky[i] > kym ? o->ky[i] : kym;
  for (int i = 0; i < o->nz / 2 + 1; ++i) kzm = o->kz[i] > kzm ? o->kz[i] : kzm;
  double k[3] = {kxm, kym, kzm};
  return norm2_3(k);
}

/* nq, ReadCLuc.hpp:65 */
int mdfto_nq_for_dq(const mdft_oracle* o, double dq) {
  return (int)(mdfto_qmax(o) / dq + 0.5) + 2;
}

/* Luc reorder + sign fold, MDFT_Convolution.hpp:239-311 (with the 5-D
 * projection index of ReadCLuc.hpp:88-103). */
int mdfto_set_luc(mdft_oracle* o, const int* luc_index, const double* luc,
                  int np_luc, int nq, double dq) {
  int mmax = o->mmax, mrso = o->mrso;
  int K = mmax / mrso;
  int npm = 2 * mmax / mrso + 1;
  int m2 = 2 * mmax + 1;
  int need = mdfto_nq_for_dq(o, dq);
  if (nq < need) return 1;
  /* The reader keeps exactly `need` rows; `stride` is the caller's row
   * length. */
  const int stride = nq;
  nq = need;
  int* p5 = (int*)calloc((size_t)(mmax + 1) * (mmax + 1) * npm * npm * m2, sizeof(int));
#define P5(a, b, c, d, e) p5[((((a) * (mmax + 1) + (b)) * npm + (c)) * npm + (d)) * m2 + (e)]
  for (int ip = 0; ip < np_luc; ip++) {
    int im = luc_index[0 * np_luc + ip], in = luc_index[1 * np_luc + ip];
    int imu = luc_index[2 * np_luc + ip], inu = luc_index[3 * np_luc + ip];
    int ikhi = luc_index[4 * np_luc + ip];
    if (im < 0 || im > mmax || in < 0 || in > mmax) continue;
    int c2 = imu / mrso + K, d2 = inu / mrso + K, e2 = ikhi + mmax;
    if (c2 < 0 || c2 >= npm || d2 < 0 || d2 >= npm || e2 < 0 || e2 >= m2) continue;
    P5(im, in, c2, d2, e2) = ip;
  }
  int np_new = o->np_new;
  free(o->mnmunukhi_q);
  o->mnmunukhi_q = (cplx*)malloc(sizeof(cplx) * (size_t)np_new * nq);
  const cplx* L = (const cplx*)luc;
  int* n_new = (int*)malloc(sizeof(int) * np_new);
  int* nu_new = (int*)malloc(sizeof(int) * np_new);
  int* khi_new = (int*)malloc(sizeof(int) * np_new);
  int i = 0;
  for (int im = 0; im <= mmax; ++im)
    for (int ikhi = -im; ikhi <= im; ++ikhi)
      for (int imu2 = 0; imu2 <= im / mrso; ++imu2)
        for (int in = abs(ikhi); in <= mmax; ++in)
          for (int inu2 = -in / mrso; inu2 <= in / mrso; ++inu2) {
            n_new[i] = in;
            nu_new[i] = inu2 * mrso;
            khi_new[i] = ikhi;
            int ip = P5(im, in, imu2 + K, inu2 + K, ikhi + mmax);
            for (int iq = 0; iq < nq; iq++)
              o->mnmunukhi_q[(size_t)i * nq + iq] = L[(size_t)ip * stride + iq];
            i++;
          }
#undef P5
  for (int ip = 0; ip < np_new; ip++) {
    double s;
    if (nu_new[ip] < 0)
      s = pow(-1.0, (double)(khi_new[ip] + nu_new[ip]));
    else
      s = pow(-1.0, (double)n_new[ip]);
    for (int iq = 0; iq < nq; iq++) {
      cplx* z = &o->mnmunukhi_q[(size_t)ip * nq + iq];
      *z = cscale(*z, s);
    }
  }
  free(n_new);
  free(nu_new);
  free(khi_new);
  free(p5);
  o->nq = nq;
  o->dq = dq;
  return 0;
}

void mdfto_gamma_p_map(const mdft_oracle* o, int* map) {
  memcpy(map, o->gamma_p_map, sizeof(int) * 3 * (size_t)o->npairs);
}
void mdfto_ia_map(const mdft_oracle* o, int* ia) {
  int n2 = 2 * o->mmax / o->mrso + 1;
  memcpy(ia, o->ia_map, sizeof(int) * (size_t)o->np * (o->mmax + 1) * n2);
}
void mdfto_mnmunukhi_q(const mdft_oracle* o, double* tab) {
  memcpy(tab, o->mnmunukhi_q, sizeof(cplx) * (size_t)o->np_new * o->nq);
}

/* ------------------------------------------------------------------------ */
/* Stages                                                                     */
/* ------------------------------------------------------------------------ */

/* get_delta_rho, MDFT_Solvent.hpp:578-596 */
void mdfto_delta_rho(const double* xi, double* dr, size_t n, double rho0) {
#pragma omp parallel for schedule(static)
  for (long i = 0; i < (long)n; ++i) dr[i] = rho0 * (xi[i] * xi[i] - 1.0);
}

/* angl2proj, MDFT_OrientationProjectionTransform.hpp:270-380.
 * rfft2 over (phi, psi) with no normalisation, then the conj/shift of
 * :329-355 and the theta contraction of :359-378. */
void mdfto_angl2proj(const mdft_oracle* o, const double* orient, double* proj) {
  const int nt = o->ntheta, nphi = o->nphi, npsi = o->npsi, mmax = o->mmax;
  const int K = mmax / o->mrso, np = o->np;
  const long N = (long)o->nx * o->ny * o->nz;
  cplx* P = (cplx*)proj;
  cplx* twphi = (cplx*)malloc(sizeof(cplx) * nphi);
  cplx* twpsi = (cplx*)malloc(sizeof(cplx) * npsi);
  for (int t = 0; t < nphi; ++t) {
    long double a = 2.0L * kPiL * t / nphi;
    twphi[t] = cx((double)cosl(a), -(double)sinl(a));
  }
  for (int t = 0; t < npsi; ++t) {
    long double a = 2.0L * kPiL * t / npsi;
    twpsi[t] = cx((double)cosl(a), -(double)sinl(a));
  }
  const double nrm = (double)(nphi * npsi);
#pragma omp parallel
  {
    cplx* Y = (cplx*)malloc(sizeof(cplx) * nphi * (K + 1));
    cplx* sf = (cplx*)malloc(sizeof(cplx) * nt * nphi * (K + 1));
#pragma omp for schedule(static)
    for (long r = 0; r < N; ++r) {
      const double* orr = orient + r * (long)o->no;
      for (int it = 0; it < nt; ++it) {
        const double* ot = orr + it * nphi * npsi;
        /* psi-direction real DFT for kpsi = 0..K */
        for (int iphi = 0; iphi < nphi; ++iphi)
          for (int kp = 0; kp <= K; ++kp) {
            cplx acc = cx(0, 0);
            for (int ipsi = 0; ipsi < npsi; ++ipsi)
              acc = cadd(acc, cscale(twpsi[(kp * ipsi) % npsi], ot[iphi * npsi + ipsi]));
            Y[iphi * (K + 1) + kp] = acc;
          }
        /* phi-direction complex DFT; s_f(mup + mmax) = conj(ohat(mup mod nphi)) / nrm */
        for (int kf = 0; kf < nphi; ++kf)
          for (int kp = 0; kp <= K; ++kp) {
            cplx acc = cx(0, 0);
            for (int iphi = 0; iphi < nphi; ++iphi)
              acc = cadd(acc, cmul(Y[iphi * (K + 1) + kp], twphi[(kf * iphi) % nphi]));
            int mup = kf <= mmax ? kf : kf - nphi;
            cplx s = cconj(acc);
            s.re = s.re / nrm;
            s.im = s.im / nrm;
            sf[(it * nphi + (mup + mmax)) * (K + 1) + kp] = s;
          }
      }
      for (int ip = 0; ip < np; ++ip) {
        int m = o->pm[ip], mup = o->pmup[ip], mu2 = o->pmu2[ip];
        cplx sum = cx(0, 0);
        for (int it = 0; it < nt; ++it) {
          cplx t = sf[(it * nphi + (mup + mmax)) * (K + 1) + mu2];
          t = cscale(t, o->wigner[it * np + ip]);
          t = cscale(t, o->wthetaofntheta[it]);
          t = cscale(t, o->fm[m]);
          sum = cadd(sum, t);
        }
        P[(long)ip * N + r] = sum;
      }
    }
    free(Y);
    free(sf);
  }
  free(twphi);
  free(twpsi);
}

/* proj2angl, MDFT_OrientationProjectionTransform.hpp:391-484.
 * The synthesis of :435-449, the scatter of :454-477, then an unnormalised
 * 2-D C2R transform (imaginary part of each kpsi=0 column sum discarded, the
 * FFTW/cuFFT/numpy convention for odd npsi). */
void mdfto_proj2angl(const mdft_oracle* o, const double* proj, double* orient) {
  const int nt = o->ntheta, nphi = o->nphi, npsi = o->npsi, mmax = o->mmax;
  const int mrso = o->mrso, K = mmax / mrso, np = o->np;
  const long N = (long)o->nx * o->ny * o->nz;
  const cplx* P = (const cplx*)proj;
  cplx* twphi = (cplx*)malloc(sizeof(cplx) * nphi);
  cplx* twpsi = (cplx*)malloc(sizeof(cplx) * npsi);
  for (int t = 0; t < nphi; ++t) {
    long double a = 2.0L * kPiL * t / nphi;
    twphi[t] = cx((double)cosl(a), (double)sinl(a));
  }
  for (int t = 0; t < npsi; ++t) {
    long double a = 2.0L * kPiL * t / npsi;
    twpsi[t] = cx((double)cosl(a), (double)sinl(a));
  }
  const int m2 = 2 * mmax + 1;
#pragma omp parallel
  {
    cplx* sf = (cplx*)malloc(sizeof(cplx) * m2 * (K + 1));
    cplx* oh = (cplx*)malloc(sizeof(cplx) * nphi * (K + 1));
    cplx* U = (cplx*)malloc(sizeof(cplx) * nphi * (K + 1));
#pragma omp for schedule(static)
    for (long r = 0; r < N; ++r) {
      for (int it = 0; it < nt; ++it) {
        for (int imup = 0; imup < m2; ++imup)
          for (int imu2 = 0; imu2 <= K; ++imu2) {
            cplx sum = cx(0, 0);
            int a = abs(imup - mmax), b = mrso * abs(imu2);
            int m_init = a > b ? a : b;
            for (int im = m_init; im <= mmax; ++im) {
              int ip = o->pmap[(im * m2 + imup) * (K + 1) + imu2];
              cplx t = cscale(P[(long)ip * N + r], o->wigner[it * np + ip]);
              t = cscale(t, o->fm[im]);
              sum = cadd(sum, t);
            }
            sf[imup * (K + 1) + imu2] = cconj(sum);
          }
        /* scatter to FFT order */
        for (int kf = 0; kf < nphi; ++kf)
          for (int kp = 0; kp <= K; ++kp) {
            int mup = kf <= mmax ? kf : kf - nphi;
            oh[kf * (K + 1) + kp] = sf[(mup + mmax) * (K + 1) + kp];
          }
        /* inverse complex DFT along phi */
        for (int iphi = 0; iphi < nphi; ++iphi)
          for (int kp = 0; kp <= K; ++kp) {
            cplx acc = cx(0, 0);
            for (int kf = 0; kf < nphi; ++kf)
              acc = cadd(acc, cmul(oh[kf * (K + 1) + kp], twphi[(kf * iphi) % nphi]));
            U[iphi * (K + 1) + kp] = acc;
          }
        /* C2R along psi (npsi odd) */
        double* out = orient + r * (long)o->no + it * nphi * npsi;
        for (int iphi = 0; iphi < nphi; ++iphi)
          for (int ipsi = 0; ipsi < npsi; ++ipsi) {
            double v = U[iphi * (K + 1) + 0].re;
            for (int kp = 1; kp <= K; ++kp) {
              cplx t = cmul(U[iphi * (K + 1) + kp], twpsi[(kp * ipsi) % npsi]);
              v += 2.0 * t.re;
            }
            out[iphi * npsi + ipsi] = v;
          }
      }
    }
    free(sf);
    free(oh);
    free(U);
  }
  free(twphi);
  free(twpsi);
}

/* Convolution::execute, MDFT_Convolution.hpp:326-548 */
void mdfto_conv_execute(const mdft_oracle* o, double* proj) {
  const int nx = o->nx, ny = o->ny, nz = o->nz, np = o->np;
  const int mmax = o->mmax, mrso = o->mrso, K = mmax / mrso;
  const int m2 = 2 * mmax + 1, n2 = 2 * mmax / mrso + 1;
  const long N = (long)nx * ny * nz;
  const double eps = 2.220446049250313e-16;
  cplx* P = (cplx*)proj;
  mdfto_fft3d(proj, np, nx, ny, nz, -1);
#define PMAP(m, mup, mu2) o->pmap[((m) * m2 + (mup)) * (K + 1) + (mu2)]
#pragma omp parallel
  {
    cplx* R = (cplx*)calloc((size_t)(mmax + 1) * m2 * m2, sizeof(cplx));
    cplx* gq = (cplx*)malloc(sizeof(cplx) * np);
    cplx* gmq = (cplx*)malloc(sizeof(cplx) * np);
    cplx* dq_ = (cplx*)malloc(sizeof(cplx) * np);
    cplx* dmq = (cplx*)malloc(sizeof(cplx) * np);
    cplx* ceff = (cplx*)malloc(sizeof(cplx) * o->np_new);
#pragma omp for schedule(dynamic, 64)
    for (long idx = 0; idx < o->npairs; ++idx) {
      const int ix = o->gamma_p_map[3 * idx], iy = o->gamma_p_map[3 * idx + 1],
                iz = o->gamma_p_map[3 * idx + 2];
      double q[3] = {o->kx[ix], o->ky[iy], o->kz[iz]};
      const int ixm = inv_index(ix, nx), iym = inv_index(iy, ny), izm = inv_index(iz, nz);
      rotation_matrix(q, mmax, o->rot_a, o->rot_b, o->rot_c, o->rot_d, R);
#define RR(l, i, j) R[((l) * m2 + (i)) * m2 + (j)]
      const long lq = ((long)ix * ny + iy) * nz + iz;
      const long lmq = ((long)ixm * ny + iym) * nz + izm;
      for (int ip = 0; ip < np; ++ip) {
        gq[ip] = P[(long)ip * N + lq];
        gmq[ip] = P[(long)ip * N + lmq];
      }
      /* rotation to the q frame, :427-443 */
      for (int ip = 0; ip < np; ++ip) {
        int im = o->pm[ip], ikhi = o->pmup[ip], imu2 = o->pmu2[ip];
        cplx a = cx(0, 0), b = cx(0, 0);
        for (int imup = -im; imup <= im; imup++) {
          int ipm = PMAP(im, imup + mmax, imu2);
          a = cadd(a, cmul(gq[ipm], RR(im, imup + mmax, ikhi + mmax)));
          b = cadd(b, cmul(gmq[ipm], RR(im, imup + mmax, -ikhi + mmax)));
        }
        dq_[ip] = a;
        dmq[ip] = cscale(b, (im % 2 == 0) ? 1.0 : -1.0);
      }
      /* interpolation of c(|q|), :449-463 */
      double effectiveiq = norm2_3(q) / o->dq;
      int iq = (int)effectiveiq;
      double alpha = effectiveiq - (double)iq;
      for (int i = 0; i < o->np_new; ++i) {
        cplx lo = o->mnmunukhi_q[(size_t)i * o->nq + iq];
        cplx hi = o->mnmunukhi_q[(size_t)i * o->nq + iq + 1];
        ceff[i] = cadd(cscale(hi, alpha), cscale(lo, 1.0 - alpha));
      }
      /* Ornstein-Zernike in the molecular frame, :468-496 */
      for (int ip = 0; ip < np; ++ip) {
        int ikhi = o->pmup[ip];
        cplx sq = cx(0, 0), smq = cx(0, 0);
        for (int in = abs(ikhi); in <= mmax; in++)
          for (int inu2 = -in / mrso; inu2 <= in / mrso; inu2++) {
            int ia = o->ia_map[(ip * (mmax + 1) + in) * n2 + inu2 + mmax / mrso];
            cplx c = ceff[ia];
            if (inu2 < 0) {
              int ipm = PMAP(in, ikhi + mmax, abs(inu2));
              sq = cadd(sq, cmul(c, dq_[ipm]));
              smq = cadd(smq, cmul(c, dmq[ipm]));
            } else {
              int ipm = PMAP(in, ikhi + mmax, inu2);
              sq = cadd(sq, cmul(c, cconj(dmq[ipm])));
              smq = cadd(smq, cmul(c, cconj(dq_[ipm])));
            }
          }
        gq[ip] = sq;
        gmq[ip] = smq;
      }
      /* underflow chop of gamma (all of it first), :514-517 */
      for (int ip = 0; ip < np; ++ip) {
        gq[ip] = prevent_underflow(gq[ip], eps);
        gmq[ip] = prevent_underflow(gmq[ip], eps);
      }
      const int qeq = (ixm == ix && iym == iy && izm == iz);
      const int singular = qeq && (ix == nx / 2 || iy == ny / 2 || iz == nz / 2);
      /* rotation back to the fixed frame and stores, :518-541 */
      for (int ip = 0; ip < np; ++ip) {
        int im = o->pm[ip], imup = o->pmup[ip], imu2 = o->pmu2[ip];
        cplx a = cx(0, 0), b = cx(0, 0);
        for (int ikhi = -im; ikhi <= im; ikhi++) {
          int ipm = PMAP(im, ikhi + mmax, imu2);
          a = cadd(a, cmul(gq[ipm], cconj(RR(im, imup + mmax, ikhi + mmax))));
          b = cadd(b, cmul(gmq[ipm], cconj(RR(im, imup + mmax, -ikhi + mmax))));
        }
        b = cscale(b, (im % 2 == 0) ? 1.0 : -1.0);
        P[(long)ip * N + lq] = a;
        P[(long)ip * N + lmq] = singular ? cconj(b) : b;
      }
#undef RR
    }
    free(R);
    free(gq);
    free(gmq);
    free(dq_);
    free(dmq);
    free(ceff);
  }
#undef PMAP
  mdfto_fft3d(proj, np, nx, ny, nz, +1);
}

/* get_delta_f, MDFT_Solvent.hpp:617-660.  The per-point sum over
 * orientations runs in index order as in the serial backend; the sum over
 * points is compensated (Neumaier) so that the oracle gives the exact-rounded
 * total, independent of any parallel reduction order. */
double mdfto_delta_f(const double* xi, const double* vexc, const double* w,
                     double* delta_f, size_t nxyz, int no, double rho0,
                     double prefactor) {
  double* part = (double*)malloc(sizeof(double) * nxyz);
#pragma omp parallel for schedule(static)
  for (long r = 0; r < (long)nxyz; ++r) {
    double sum = 0;
    for (int io = 0; io < no; ++io) {
      size_t i = (size_t)r * no + io;
      sum += vexc[i] * w[io] * (xi[i] * xi[i] - 1.0);
      delta_f[i] = 2.0 * rho0 * xi[i] * vexc[i];
    }
    part[r] = rho0 * sum * prefactor;
  }
  double s = 0.0, c = 0.0;
  for (size_t r = 0; r < nxyz; ++r) {
    double t = s + part[r];
    if (fabs(s) >= fabs(part[r]))
      c += (s - t) + part[r];
    else
      c += (part[r] - t) + s;
    s = t;
  }
  free(part);
  return s + c;
}

/* Solvents::m_prefactor, MDFT_Solvent.hpp:366-368 with kT of
 * MDFT_Thermo.hpp:60 and the constants of MDFT_Constants.hpp. */
double mdfto_prefactor(double temperature, int mrso, double n0) {
  const double boltz = 1.38064852e-23, navo = 6.02214129e23;
  const double pi = 3.14159265358979323846;
  double kbt = boltz * navo * temperature * 1e-3;
  return -2 * kbt * 4 * pi * pi / mrso / n0;
}
