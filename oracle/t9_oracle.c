/*
 * FP64 CPU oracle for the AMOEBA mutual-polarization path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker: tests, the smoke entry
 * and the CPU-baseline leg of the benchmark call it; the product (the CUDA
 * library under tinker-gpu_gb300/csrc) never links or calls it.
 *
 * It restates, in double precision, the algorithms of Tinker9 (tinker-gpu):
 *   - multipole frame rotation         include/seq/rotpole.h:7-224
 *   - Thole damping                    include/seq/damp.h:8-44
 *   - Ewald damping b_n recursion      include/seq/damp.h:136-151
 *   - real-space d/p field pair        include/seq/pair_field.h:127-256
 *   - real-space mutual field pair     include/seq/pair_field.h:333-420
 *   - exclusion-pair semantics         src/amoeba/epolar.cpp:88-484,
 *                                      src/cu/amoeba/ufield_cu1.cc:29-96
 *   - B-spline weights                 include/seq/bsplgen.h:27-116
 *   - PME spreading / gather           src/cu/pme.cu:14-255, :383-870
 *   - reciprocal convolution           src/cu/pme.cu:908-1031
 *   - Cartesian<->fractional frames    src/cu/pme.cu:1052-1300
 *   - recip/self field terms           src/cu/amoeba/field.cu:12-33, :71-118
 *   - sparse preconditioner            src/cu/amoeba/precond.cu:12-43,
 *                                      src/cu/amoeba/sparsePrecond_cu1.cc:60-120
 *   - PCG control flow                 src/cu/amoeba/pcg.cu:14-185,
 *                                      src/cu/induce.cu:17-232
 *   - ASPC extrapolation               src/cu/upredict.cu:34-130
 * The B-spline moduli follow Essmann et al., J. Chem. Phys. 103, 8577 (1995)
 * with Tinker's published "optimal zeta" Euler-spline correction (the
 * reference obtains them from Fortran dftmod/bspline, src/pme.cpp:84-117).
 * erfc in double precision is 1 - erf(x), as the reference's double build
 * defines it (include/math/libfunc.h:76-77).
 *
 * Parity pins: tests/golden holds the reference's own known answers for the
 * 22-atom local-frame case (test/localframe.cpp) and four more reference
 * tests; oracle/ref_harness.cpp runs the reference's own pair, frame and
 * B-spline routines compiled from its source (oracle/build_ref.py), and
 * tests/test_oracle_reference_build.py compares this file with them.
 */
#include <complex.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define OR_PI 3.14159265358979323846
#define OR_SQRTPI 1.77245385090551602730

typedef struct {
   int n;
   const double* x;
   const double* y;
   const double* z;
   const double* rpole;     /* [n][10]: q, dx, dy, dz, qxx, qyy, qzz, qxy, qxz, qyz */
   const double* polarity;  /* [n] */
   const double* thole;     /* [n] */
   const double* pdamp;     /* [n] */
   int nexcl;               /* scaled pairs, i < k */
   const int* excl_ik;      /* [nexcl][2] */
   const double* excl_scale;/* [nexcl][4]: m, d, p, u */
   int periodic;            /* orthorhombic box when 1 */
   double box[3];
   int use_ewald;
   double aewald;
   int nfft[3];
   int bsorder;
   double cutoff;           /* real-space cutoff (Ewald) or multipole cutoff */
   double electric;
   int nthl;                /* > 0: per-type-pair Thole table (jpolar / thlval) */
   const int* ptype;        /* [n] polarization type, 0..nthl-1 */
   const double* thl;       /* [nthl][nthl] */
   double exfld[3];         /* uniform external field, e/A^2 (zero: none) */
   int real_only;           /* 1: dfield / ufield leave out the reciprocal and self terms */
} or_system;

typedef struct {
   double poleps;         /* RMS residual threshold, Debye */
   int politer;           /* iteration cap */
   double pcgpeek;
   double udiag;          /* diagonal weight of the sparse preconditioner */
   int pcgprec;           /* 1: sparse preconditioner, 0: diagonal */
   double precond_cutoff; /* usolve cutoff + list buffer */
   int guess;             /* 0 zero, 1 direct (alpha E), 2 caller-supplied */
   double debye;
} or_induce_opts;

int or_nthreads(void)
{
#ifdef _OPENMP
   return omp_get_max_threads();
#else
   return 1;
#endif
}

void or_set_threads(int t)
{
#ifdef _OPENMP
   if (t > 0)
      omp_set_num_threads(t);
#else
   (void)t;
#endif
}

/* ------------------------------------------------------------------ */
/* geometry                                                            */

static inline void or_image(const or_system* s, double* xr, double* yr, double* zr)
{
   if (!s->periodic)
      return;
   *xr -= s->box[0] * nearbyint(*xr / s->box[0]);
   *yr -= s->box[1] * nearbyint(*yr / s->box[1]);
   *zr -= s->box[2] * nearbyint(*zr / s->box[2]);
}

/* Half pair list (i < k, r <= cut) built with cells; all pairs if the box is
 * too small for three cells per side or the system is not periodic. */
typedef struct {
   int npair;
   int* ik;
} or_pairs;

static void or_pairs_free(or_pairs* p)
{
   free(p->ik);
   p->ik = NULL;
   p->npair = 0;
}

static void or_pairs_push(or_pairs* p, int* cap, int i, int k)
{
   if (p->npair == *cap) {
      *cap = *cap ? 2 * *cap : 1024;
      p->ik = (int*)realloc(p->ik, sizeof(int) * 2 * (size_t)(*cap));
   }
   p->ik[2 * p->npair] = i < k ? i : k;
   p->ik[2 * p->npair + 1] = i < k ? k : i;
   p->npair++;
}

static int cmp_pair(const void* a, const void* b)
{
   const int* p = (const int*)a;
   const int* q = (const int*)b;
   if (p[0] != q[0])
      return p[0] < q[0] ? -1 : 1;
   if (p[1] != q[1])
      return p[1] < q[1] ? -1 : 1;
   return 0;
}

static void or_build_pairs(const or_system* s, double cut, or_pairs* out)
{
   const int n = s->n;
   const double cut2 = cut * cut;
   int cap = 0;
   out->npair = 0;
   out->ik = NULL;
   int nc[3] = {0, 0, 0};
   int usecell = s->periodic;
   if (usecell) {
      for (int d = 0; d < 3; ++d) {
         nc[d] = (int)floor(s->box[d] / cut);
         if (nc[d] < 3)
            usecell = 0;
      }
   }
   if (!usecell) {
      for (int i = 0; i < n; ++i)
         for (int k = i + 1; k < n; ++k) {
            double xr = s->x[k] - s->x[i], yr = s->y[k] - s->y[i], zr = s->z[k] - s->z[i];
            or_image(s, &xr, &yr, &zr);
            if (xr * xr + yr * yr + zr * zr <= cut2)
               or_pairs_push(out, &cap, i, k);
         }
      return;
   }
   const int ncell = nc[0] * nc[1] * nc[2];
   int* head = (int*)malloc(sizeof(int) * ncell);
   int* next = (int*)malloc(sizeof(int) * n);
   int* cid = (int*)malloc(sizeof(int) * 3 * n);
   for (int c = 0; c < ncell; ++c)
      head[c] = -1;
   for (int i = 0; i < n; ++i) {
      double p[3] = {s->x[i], s->y[i], s->z[i]};
      int c3[3];
      for (int d = 0; d < 3; ++d) {
         double f = p[d] / s->box[d];
         f -= floor(f);
         int c = (int)(f * nc[d]);
         if (c >= nc[d])
            c = nc[d] - 1;
         c3[d] = c;
         cid[3 * i + d] = c;
      }
      int c = (c3[2] * nc[1] + c3[1]) * nc[0] + c3[0];
      next[i] = head[c];
      head[c] = i;
   }
   for (int i = 0; i < n; ++i) {
      for (int dz = -1; dz <= 1; ++dz)
         for (int dy = -1; dy <= 1; ++dy)
            for (int dx = -1; dx <= 1; ++dx) {
               int cx = (cid[3 * i] + dx + nc[0]) % nc[0];
               int cy = (cid[3 * i + 1] + dy + nc[1]) % nc[1];
               int cz = (cid[3 * i + 2] + dz + nc[2]) % nc[2];
               for (int k = head[(cz * nc[1] + cy) * nc[0] + cx]; k >= 0; k = next[k]) {
                  if (k <= i)
                     continue;
                  double xr = s->x[k] - s->x[i], yr = s->y[k] - s->y[i], zr = s->z[k] - s->z[i];
                  or_image(s, &xr, &yr, &zr);
                  if (xr * xr + yr * yr + zr * zr <= cut2)
                     or_pairs_push(out, &cap, i, k);
               }
            }
   }
   free(head);
   free(next);
   free(cid);
   qsort(out->ik, out->npair, 2 * sizeof(int), cmp_pair);
}

/* Per-atom CSR of scaled pairs for lookup by (i, k). */
typedef struct {
   int* start;
   int* kk;
   const double* sc[1];
   int* idx;
} or_excl;

static void or_excl_build(const or_system* s, or_excl* e)
{
   const int n = s->n;
   e->start = (int*)calloc(n + 1, sizeof(int));
   e->kk = (int*)malloc(sizeof(int) * (s->nexcl + 1));
   e->idx = (int*)malloc(sizeof(int) * (s->nexcl + 1));
   for (int j = 0; j < s->nexcl; ++j)
      e->start[s->excl_ik[2 * j] + 1]++;
   for (int i = 0; i < n; ++i)
      e->start[i + 1] += e->start[i];
   int* fill = (int*)calloc(n, sizeof(int));
   for (int j = 0; j < s->nexcl; ++j) {
      int i = s->excl_ik[2 * j];
      int pos = e->start[i] + fill[i]++;
      e->kk[pos] = s->excl_ik[2 * j + 1];
      e->idx[pos] = j;
   }
   free(fill);
}

static void or_excl_free(or_excl* e)
{
   free(e->start);
   free(e->kk);
   free(e->idx);
}

/* scales m, d, p, u for pair i < k; all 1 when the pair is not listed */
static inline void or_excl_get(const or_system* s, const or_excl* e, int i, int k, double sc[4])
{
   sc[0] = sc[1] = sc[2] = sc[3] = 1;
   for (int j = e->start[i]; j < e->start[i + 1]; ++j)
      if (e->kk[j] == k) {
         const double* v = &s->excl_scale[4 * e->idx[j]];
         sc[0] = v[0];
         sc[1] = v[1];
         sc[2] = v[2];
         sc[3] = v[3];
         return;
      }
}

/* ------------------------------------------------------------------ */
/* damping (include/seq/damp.h)                                        */

/* Thole coefficient of pair (i, k): thlval[jpolar_i][jpolar_k] when a table
 * is set (src/cu/amoeba/ufield_cu1.cc, dfield_cu1.cc, sparsePrecond_cu1.cc,
 * epolar_cu1.cc), else min(thole_i, thole_k) (damp_thole2/3, damp.h:19-44).
 * Passed as both pti and ptk to the pair routines below. */
static inline double or_pair_gamma(const or_system* s, int i, int k)
{
   if (s->nthl > 0)
      return s->thl[s->ptype[i] * s->nthl + s->ptype[k]];
   return fmin(s->thole[i], s->thole[k]);
}

static inline void or_thole3(double r, double pdi, double pti, double pdk, double ptk, double* s3, double* s5,
   double* s7)
{
   double pgamma = fmin(pti, ptk);
   double damp = pdi * pdk;
   double ratio = r / damp;
   damp = (damp == 0 ? -1.0e16 : -pgamma * ratio * ratio * ratio);
   double ex = exp(damp);
   *s3 = 1 - ex;
   *s5 = 1 - ex * (1 - damp);
   if (s7)
      *s7 = 1 - ex * (1 - damp + 0.6 * damp * damp);
}

static inline void or_ewald_bn(int order, double* bn, double r, double rr2, double aewald)
{
   double ralpha = aewald * r;
   bn[0] = (1.0 - erf(ralpha)) / r;
   double alsq2 = 2 * aewald * aewald;
   double alsq2n = 1.0 / (OR_SQRTPI * aewald);
   double exp2a = exp(-ralpha * ralpha);
   for (int j = 1; j < order; ++j) {
      alsq2n *= alsq2;
      bn[j] = ((j + j - 1) * bn[j - 1] + alsq2n * exp2a) * rr2;
   }
}

/* ------------------------------------------------------------------ */
/* frame rotation (include/seq/rotpole.h)                              */

enum { LF_NONE = 0, LF_Z_ONLY = 1, LF_Z_THEN_X = 2, LF_BISECTOR = 3, LF_Z_BISECT = 4, LF_3_FOLD = 5 };

static void or_norm(double* a)
{
   double r = 1.0 / sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
   a[0] *= r;
   a[1] *= r;
   a[2] *= r;
}

/* Local frame of atom i: rows of a[3][3] are the x, y, z axes in the global
 * frame (rotpole.h:52-118). */
static void or_frame_matrix(int i, const int* frames, const double* x, const double* y, const double* z,
   double a[3][3])
{
   int iz = frames[4 * i], ix = frames[4 * i + 1], iyy = frames[4 * i + 2], ax = frames[4 * i + 3];
   for (int r = 0; r < 3; ++r)
      for (int c = 0; c < 3; ++c)
         a[r][c] = r == c ? 1.0 : 0.0;
   if (ax != LF_NONE) {
      double *xx = a[0], *yy = a[1], *zz = a[2];
      zz[0] = x[iz] - x[i];
      zz[1] = y[iz] - y[i];
      zz[2] = z[iz] - z[i];
      or_norm(zz);
      if (ax == LF_Z_ONLY) {
         int okay = !(fabs(zz[0]) > 0.866);
         xx[0] = okay ? 1 : 0;
         xx[1] = okay ? 0 : 1;
         xx[2] = 0;
      } else {
         xx[0] = x[ix] - x[i];
         xx[1] = y[ix] - y[i];
         xx[2] = z[ix] - z[i];
         or_norm(xx);
      }
      if (ax == LF_Z_BISECT || ax == LF_3_FOLD) {
         int iy = abs(iyy) - 1;
         yy[0] = x[iy] - x[i];
         yy[1] = y[iy] - y[i];
         yy[2] = z[iy] - z[i];
         or_norm(yy);
      }
      if (ax == LF_BISECTOR) {
         for (int d = 0; d < 3; ++d)
            zz[d] += xx[d];
         or_norm(zz);
      } else if (ax == LF_Z_BISECT) {
         for (int d = 0; d < 3; ++d)
            xx[d] += yy[d];
         or_norm(xx);
      } else if (ax == LF_3_FOLD) {
         for (int d = 0; d < 3; ++d)
            zz[d] += xx[d] + yy[d];
         or_norm(zz);
      }
      double dot = xx[0] * zz[0] + xx[1] * zz[1] + xx[2] * zz[2];
      for (int d = 0; d < 3; ++d)
         xx[d] -= dot * zz[d];
      or_norm(xx);
      a[1][0] = a[0][2] * a[2][1] - a[0][1] * a[2][2];
      a[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
      a[1][2] = a[0][1] * a[2][0] - a[0][0] * a[2][1];
   }
}

/* frames of all atoms, out[n][9] (rows x, y, z axes) */
void or_frames(int n, const int* frames, const double* x, const double* y, const double* z, double* out)
{
   for (int i = 0; i < n; ++i) {
      double a[3][3];
      or_frame_matrix(i, frames, x, y, z, a);
      for (int r = 0; r < 3; ++r)
         for (int c = 0; c < 3; ++c)
            out[9 * i + 3 * r + c] = a[r][c];
   }
}

/* frames[n][4] = zaxis (0-based), xaxis (0-based), yaxis (1-based, signed), polaxe.
 * pole is modified in place by the chirality check, as the reference does. */
void or_rotpole(int n, const int* frames, double* pole, const double* x, const double* y, const double* z,
   double* rpole)
{
   for (int i = 0; i < n; ++i) {
      int iz = frames[4 * i], ix = frames[4 * i + 1], iyy = frames[4 * i + 2], ax = frames[4 * i + 3];
      /* chirality (rotpole.h:7-50) */
      if (ax == LF_Z_THEN_X && iyy != 0) {
         int id = abs(iyy) - 1;
         double xad = x[i] - x[id], yad = y[i] - y[id], zad = z[i] - z[id];
         double xbd = x[iz] - x[id], ybd = y[iz] - y[id], zbd = z[iz] - z[id];
         double xcd = x[ix] - x[id], ycd = y[ix] - y[id], zcd = z[ix] - z[id];
         double c1 = ybd * zcd - zbd * ycd, c2 = ycd * zad - zcd * yad, c3 = yad * zbd - zad * ybd;
         double vol = xad * c1 + xbd * c2 + xcd * c3;
         if ((iyy < 0 && vol > 0) || (iyy > 0 && vol < 0)) {
            pole[10 * i + 2] = -pole[10 * i + 2];
            pole[10 * i + 7] = -pole[10 * i + 7];
            pole[10 * i + 9] = -pole[10 * i + 9];
         }
      }
      double a[3][3];
      or_frame_matrix(i, frames, x, y, z, a);
      const double* p = &pole[10 * i];
      double* rp = &rpole[10 * i];
      rp[0] = p[0];
      for (int c = 1; c < 4; ++c) {
         rp[c] = 0;
         for (int j = 1; j < 4; ++j)
            rp[c] += p[j] * a[j - 1][c - 1];
      }
      double mp[3][3] = {{p[4], p[7], p[8]}, {p[7], p[5], p[9]}, {p[8], p[9], p[6]}};
      double q[3][3] = {{0}};
      for (int c = 0; c < 3; ++c)
         for (int j = 0; j <= c; ++j)
            for (int k = 0; k < 3; ++k)
               for (int m = 0; m < 3; ++m)
                  q[j][c] += a[k][c] * a[m][j] * mp[m][k];
      rp[4] = q[0][0];
      rp[5] = q[1][1];
      rp[6] = q[2][2];
      rp[7] = q[0][1];
      rp[8] = q[0][2];
      rp[9] = q[1][2];
   }
}

/* ------------------------------------------------------------------ */
/* FFT: recursive mixed radix, unnormalised, sign = -1 forward, +1 back */

static void fft_rec(const double complex* in, int istride, double complex* out, int n, int sign)
{
   if (n == 1) {
      out[0] = in[0];
      return;
   }
   int p = 0;
   for (int f = 2; f * f <= n; ++f)
      if (n % f == 0) {
         p = f;
         break;
      }
   if (p == 0)
      p = n;
   int m = n / p;
   if (m == 1) {
      for (int k = 0; k < n; ++k) {
         double complex acc = 0;
         for (int j = 0; j < n; ++j)
            acc += in[j * istride] * cexp(sign * 2.0 * OR_PI * I * (double)((long)j * k % n) / n);
         out[k] = acc;
      }
      return;
   }
   for (int r = 0; r < p; ++r)
      fft_rec(in + r * istride, istride * p, out + r * m, m, sign);
   double complex* tmp = (double complex*)malloc(sizeof(double complex) * n);
   for (int k = 0; k < m; ++k)
      for (int q = 0; q < p; ++q) {
         double complex acc = 0;
         int kk = k + q * m;
         for (int r = 0; r < p; ++r)
            acc += out[r * m + k] * cexp(sign * 2.0 * OR_PI * I * (double)((long)r * kk % n) / n);
         tmp[kk] = acc;
      }
   memcpy(out, tmp, sizeof(double complex) * n);
   free(tmp);
}

/* 3-D transform of grid[n3][n2][n1] (x fastest) */
void or_fft3d(double complex* g, int n1, int n2, int n3, int sign)
{
   int nmax = n1 > n2 ? n1 : n2;
   nmax = nmax > n3 ? nmax : n3;
#pragma omp parallel
   {
      double complex* lin = (double complex*)malloc(sizeof(double complex) * nmax);
      double complex* lout = (double complex*)malloc(sizeof(double complex) * nmax);
#pragma omp for collapse(2)
      for (int k = 0; k < n3; ++k)
         for (int j = 0; j < n2; ++j) {
            double complex* row = g + ((size_t)k * n2 + j) * n1;
            memcpy(lin, row, sizeof(double complex) * n1);
            fft_rec(lin, 1, lout, n1, sign);
            memcpy(row, lout, sizeof(double complex) * n1);
         }
#pragma omp for collapse(2)
      for (int k = 0; k < n3; ++k)
         for (int i = 0; i < n1; ++i) {
            for (int j = 0; j < n2; ++j)
               lin[j] = g[((size_t)k * n2 + j) * n1 + i];
            fft_rec(lin, 1, lout, n2, sign);
            for (int j = 0; j < n2; ++j)
               g[((size_t)k * n2 + j) * n1 + i] = lout[j];
         }
#pragma omp for collapse(2)
      for (int j = 0; j < n2; ++j)
         for (int i = 0; i < n1; ++i) {
            for (int k = 0; k < n3; ++k)
               lin[k] = g[((size_t)k * n2 + j) * n1 + i];
            fft_rec(lin, 1, lout, n3, sign);
            for (int k = 0; k < n3; ++k)
               g[((size_t)k * n2 + j) * n1 + i] = lout[k];
         }
      free(lin);
      free(lout);
   }
}

/* ------------------------------------------------------------------ */
/* PME                                                                  */

/* cardinal B-spline values at integer knots (Tinker bspline at x = 0) */
static void or_bspline_knots(int order, double* c)
{
   double x = 0;
   c[0] = 1 - x;
   c[1] = x;
   for (int k = 3; k <= order; ++k) {
      double denom = 1.0 / (k - 1);
      c[k - 1] = x * c[k - 2] * denom;
      for (int i = 1; i <= k - 2; ++i)
         c[k - i - 1] = ((x + i) * c[k - i - 2] + (k - i - x) * c[k - i - 1]) * denom;
      c[0] = (1 - x) * c[0] * denom;
   }
}

/* |b(m)|^2 moduli with the optimal-zeta correction */
void or_bsmod(int nfft, int order, double* bsmod)
{
   double* bsarray = (double*)calloc(nfft + order + 2, sizeof(double));
   double c[16];
   or_bspline_knots(order, c);
   for (int i = 0; i < order; ++i)
      bsarray[i + 1] = c[i];
   double factor = 2 * OR_PI / nfft;
   for (int i = 0; i < nfft; ++i) {
      double s1 = 0, s2 = 0;
      for (int j = 0; j < nfft; ++j) {
         double arg = factor * (double)i * (double)j;
         s1 += bsarray[j] * cos(arg);
         s2 += bsarray[j] * sin(arg);
      }
      bsmod[i] = s1 * s1 + s2 * s2;
   }
   const double eps = 1.0e-7;
   if (bsmod[0] < eps)
      bsmod[0] = 0.5 * bsmod[1];
   for (int i = 1; i < nfft - 1; ++i)
      if (bsmod[i] < eps)
         bsmod[i] = 0.5 * (bsmod[i - 1] + bsmod[i + 1]);
   if (bsmod[nfft - 1] < eps)
      bsmod[nfft - 1] = 0.5 * bsmod[nfft - 2];
   const int jcut = 50;
   for (int i = 0; i < nfft; ++i) {
      int k = i;
      if (i + 1 > nfft / 2)
         k = k - nfft;
      double zeta;
      if (k == 0)
         zeta = 1;
      else {
         double s1 = 1, s2 = 1;
         double f = OR_PI * k / nfft;
         for (int j = 1; j <= jcut; ++j) {
            double arg = f / (f + OR_PI * j);
            s1 += pow(arg, order);
            s2 += pow(arg, 2 * order);
         }
         for (int j = 1; j <= jcut; ++j) {
            double arg = f / (f - OR_PI * j);
            s1 += pow(arg, order);
            s2 += pow(arg, 2 * order);
         }
         zeta = s2 / s1;
      }
      bsmod[i] *= zeta * zeta;
   }
   free(bsarray);
}

/* B-spline weights and derivatives (bsplgen.h:27-116), theta[4*i + level] */
void or_bsplgen(double w, int order, int level, double* theta)
{
   double b[8][8];
#define BB(j, i) b[(i)-1][(j)-1]
   BB(2, 2) = w;
   BB(2, 1) = 1 - w;
   BB(3, 3) = 0.5 * w * BB(2, 2);
   BB(3, 2) = 0.5 * ((1 + w) * BB(2, 1) + (2 - w) * BB(2, 2));
   BB(3, 1) = 0.5 * (1 - w) * BB(2, 1);
   for (int i = 4; i <= order; ++i) {
      int k = i - 1;
      double denom = 1.0 / k;
      BB(i, i) = denom * w * BB(k, k);
      for (int j = 1; j <= i - 2; ++j)
         BB(i, i - j) = denom * ((w + j) * BB(k, i - j - 1) + (i - j - w) * BB(k, i - j));
      BB(i, 1) = denom * (1 - w) * BB(k, 1);
   }
   /* successive differences give the derivatives */
   for (int lv = 2; lv <= level; ++lv) {
      int k = order - lv + 1;
      for (int pass = 0; pass < lv - 1; ++pass) {
         int top = order - (lv - 2) + pass;
         BB(k, top) = BB(k, top - 1);
         for (int i = top - 1; i >= 2; --i)
            BB(k, i) = BB(k, i - 1) - BB(k, i);
         BB(k, 1) = -BB(k, 1);
      }
   }
   for (int i = 1; i <= order; ++i)
      for (int j = 1; j <= level; ++j)
         theta[4 * (i - 1) + (j - 1)] = BB(order - j + 1, i);
#undef BB
}

typedef struct {
   int n1, n2, n3, order;
   double* bsmod1;
   double* bsmod2;
   double* bsmod3;
   double complex* grid;
   double a[3][3]; /* a[f][c] = nfft_f / box_f for f == c (orthorhombic) */
} or_pme;

static void or_pme_init(const or_system* s, or_pme* p)
{
   p->n1 = s->nfft[0];
   p->n2 = s->nfft[1];
   p->n3 = s->nfft[2];
   p->order = s->bsorder;
   p->bsmod1 = (double*)malloc(sizeof(double) * p->n1);
   p->bsmod2 = (double*)malloc(sizeof(double) * p->n2);
   p->bsmod3 = (double*)malloc(sizeof(double) * p->n3);
   or_bsmod(p->n1, p->order, p->bsmod1);
   or_bsmod(p->n2, p->order, p->bsmod2);
   or_bsmod(p->n3, p->order, p->bsmod3);
   p->grid = (double complex*)malloc(sizeof(double complex) * (size_t)p->n1 * p->n2 * p->n3);
   memset(p->a, 0, sizeof(p->a));
   p->a[0][0] = p->n1 / s->box[0];
   p->a[1][1] = p->n2 / s->box[1];
   p->a[2][2] = p->n3 / s->box[2];
}

static void or_pme_free(or_pme* p)
{
   free(p->bsmod1);
   free(p->bsmod2);
   free(p->bsmod3);
   free(p->grid);
}

/* fractional position, grid origin and weights for atom i (pme.cu:31-58) */
static void or_site(const or_system* s, const or_pme* p, int i, int level, int ig[3], double th[3][20])
{
   const double pos[3] = {s->x[i], s->y[i], s->z[i]};
   const int nf[3] = {p->n1, p->n2, p->n3};
   for (int d = 0; d < 3; ++d) {
      double w = pos[d] / s->box[d];
      w = w + 0.5 - floor(w + 0.5);
      double fr = nf[d] * w;
      int g = (int)floor(fr);
      w = fr - g;
      g = g - p->order + 1;
      if (g < 0)
         g += nf[d];
      ig[d] = g;
      or_bsplgen(w, p->order, level, th[d]);
   }
}

static inline size_t or_gidx(const or_pme* p, int a, int b, int c)
{
   a = a % p->n1;
   b = b % p->n2;
   c = c % p->n3;
   return ((size_t)c * p->n2 + b) * p->n1 + a;
}

/* gridMpole: fmp[n][10] -> real part (pme.cu:103-182) */
static void or_grid_mpole(const or_system* s, or_pme* p, const double* fmp)
{
   memset(p->grid, 0, sizeof(double complex) * (size_t)p->n1 * p->n2 * p->n3);
   for (int i = 0; i < s->n; ++i) {
      int ig[3];
      double th[3][20];
      or_site(s, p, i, 3, ig, th);
      const double* f = &fmp[10 * i];
      for (int kz = 0; kz < p->order; ++kz) {
         double v0 = th[2][4 * kz], v1 = th[2][4 * kz + 1], v2 = th[2][4 * kz + 2];
         for (int jy = 0; jy < p->order; ++jy) {
            double u0 = th[1][4 * jy], u1 = th[1][4 * jy + 1], u2 = th[1][4 * jy + 2];
            double term0 = f[0] * u0 * v0 + f[2] * u1 * v0 + f[3] * u0 * v1 + f[5] * u2 * v0 + f[6] * u0 * v2
               + f[9] * u1 * v1;
            double term1 = f[1] * u0 * v0 + f[7] * u1 * v0 + f[8] * u0 * v1;
            double term2 = f[4] * u0 * v0;
            for (int ix = 0; ix < p->order; ++ix) {
               double t0 = th[0][4 * ix], t1 = th[0][4 * ix + 1], t2 = th[0][4 * ix + 2];
               p->grid[or_gidx(p, ig[0] + ix, ig[1] + jy, ig[2] + kz)] += term0 * t0 + term1 * t1 + term2 * t2;
            }
         }
      }
   }
}

/* gridUind: d -> real part, p -> imaginary part (pme.cu:185-255) */
static void or_grid_uind(const or_system* s, or_pme* p, const double* fuind, const double* fuinp)
{
   memset(p->grid, 0, sizeof(double complex) * (size_t)p->n1 * p->n2 * p->n3);
   for (int i = 0; i < s->n; ++i) {
      int ig[3];
      double th[3][20];
      or_site(s, p, i, 2, ig, th);
      const double* fd = &fuind[3 * i];
      const double* fp = &fuinp[3 * i];
      for (int kz = 0; kz < p->order; ++kz) {
         double v0 = th[2][4 * kz], v1 = th[2][4 * kz + 1];
         for (int jy = 0; jy < p->order; ++jy) {
            double u0 = th[1][4 * jy], u1 = th[1][4 * jy + 1];
            double t01 = fd[1] * u1 * v0 + fd[2] * u0 * v1, t11 = fd[0] * u0 * v0;
            double t02 = fp[1] * u1 * v0 + fp[2] * u0 * v1, t12 = fp[0] * u0 * v0;
            for (int ix = 0; ix < p->order; ++ix) {
               double t0 = th[0][4 * ix], t1 = th[0][4 * ix + 1];
               p->grid[or_gidx(p, ig[0] + ix, ig[1] + jy, ig[2] + kz)]
                  += (t01 * t0 + t11 * t1) + I * (t02 * t0 + t12 * t1);
            }
         }
      }
   }
}

/* pmeConv (pme.cu:908-1031) restricted to orthorhombic boxes; returns energy
 * 0.5 f sum G |S|^2 when f != 0 */
static double or_pme_conv(const or_system* s, or_pme* p, double f, double vir[6])
{
   const int n1 = p->n1, n2 = p->n2, n3 = p->n3;
   const double pterm = (OR_PI / s->aewald) * (OR_PI / s->aewald);
   const double volume = s->box[0] * s->box[1] * s->box[2];
   double e = 0;
   double v[6] = {0, 0, 0, 0, 0, 0};
   for (int k3 = 0; k3 < n3; ++k3)
      for (int k2 = 0; k2 < n2; ++k2)
         for (int k1 = 0; k1 < n1; ++k1) {
            size_t idx = ((size_t)k3 * n2 + k2) * n1 + k1;
            if (idx == 0) {
               p->grid[0] = 0;
               continue;
            }
            int r1 = (k1 < (n1 + 1) / 2) ? k1 : (k1 - n1);
            int r2 = (k2 < (n2 + 1) / 2) ? k2 : (k2 - n2);
            int r3 = (k3 < (n3 + 1) / 2) ? k3 : (k3 - n3);
            double h1 = r1 / s->box[0], h2 = r2 / s->box[1], h3 = r3 / s->box[2];
            double hsq = h1 * h1 + h2 * h2 + h3 * h3;
            double term = -pterm * hsq;
            double expterm = 0;
            if (term > -50) {
               double denom = hsq * OR_PI * volume * p->bsmod1[k1] * p->bsmod2[k2] * p->bsmod3[k3];
               expterm = exp(term) / denom;
               double gx = creal(p->grid[idx]), gy = cimag(p->grid[idx]);
               double eterm = 0.5 * f * expterm * (gx * gx + gy * gy);
               e += eterm;
               if (vir) {
                  double vterm = (2 / hsq) * (1 - term) * eterm;
                  v[0] += h1 * h1 * vterm - eterm;
                  v[1] += h1 * h2 * vterm;
                  v[2] += h1 * h3 * vterm;
                  v[3] += h2 * h2 * vterm - eterm;
                  v[4] += h2 * h3 * vterm;
                  v[5] += h3 * h3 * vterm - eterm;
               }
            }
            p->grid[idx] *= expterm;
         }
   if (vir)
      for (int j = 0; j < 6; ++j)
         vir[j] = v[j];
   return e;
}

/* derivative orders (t,u,v) of the 20 fphi components (pme.cu:470-640) */
static const int or_tuv[20][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {2, 0, 0}, {0, 2, 0}, {0, 0, 2},
   {1, 1, 0}, {1, 0, 1}, {0, 1, 1}, {3, 0, 0}, {0, 3, 0}, {0, 0, 3}, {2, 1, 0}, {2, 0, 1}, {1, 2, 0}, {0, 2, 1},
   {1, 0, 2}, {0, 1, 2}, {1, 1, 1}};

/* gather ncomp fractional potential components from the real (part=0) or
 * imaginary (part=1) grid into phi[n][stride] */
static void or_fphi(const or_system* s, const or_pme* p, int part, int ncomp, double* phi, int stride)
{
#pragma omp parallel for
   for (int i = 0; i < s->n; ++i) {
      int ig[3];
      double th[3][20];
      or_site(s, p, i, 4, ig, th);
      double acc[20] = {0};
      for (int kz = 0; kz < p->order; ++kz)
         for (int jy = 0; jy < p->order; ++jy)
            for (int ix = 0; ix < p->order; ++ix) {
               double complex q = p->grid[or_gidx(p, ig[0] + ix, ig[1] + jy, ig[2] + kz)];
               double g = part ? cimag(q) : creal(q);
               for (int c = 0; c < ncomp; ++c)
                  acc[c] += g * th[0][4 * ix + or_tuv[c][0]] * th[1][4 * jy + or_tuv[c][1]]
                     * th[2][4 * kz + or_tuv[c][2]];
            }
      for (int c = 0; c < ncomp; ++c)
         phi[(size_t)stride * i + c] = acc[c];
   }
}

/* Cartesian multipoles (cmp: quadrupole off-diagonals doubled) -> fractional */
static void or_cmp_to_fmp(const or_pme* p, int n, const double* rpole, double* fmp)
{
   static const int qi1[6] = {0, 1, 2, 0, 0, 1};
   static const int qi2[6] = {0, 1, 2, 1, 2, 2};
   double a[3][3];
   /* a[c][f] convention of cmpToFmp_cu1: a[k][j] = nfft_j * recip_j[k] */
   for (int c = 0; c < 3; ++c)
      for (int f = 0; f < 3; ++f)
         a[c][f] = p->a[f][c];
   double ctf6[6][6];
   for (int i1 = 0; i1 < 3; ++i1) {
      int k = qi1[i1];
      for (int i2 = 0; i2 < 6; ++i2)
         ctf6[i2][i1] = a[qi1[i2]][k] * a[qi2[i2]][k];
   }
   for (int i1 = 3; i1 < 6; ++i1) {
      int k = qi1[i1], m = qi2[i1];
      for (int i2 = 0; i2 < 6; ++i2) {
         int ii = qi1[i2], jj = qi2[i2];
         ctf6[i2][i1] = a[ii][k] * a[jj][m] + a[jj][k] * a[ii][m];
      }
   }
   for (int at = 0; at < n; ++at) {
      const double* r = &rpole[10 * at];
      double cmp[10] = {r[0], r[1], r[2], r[3], r[4], r[5], r[6], 2 * r[7], 2 * r[8], 2 * r[9]};
      double* f = &fmp[10 * at];
      f[0] = cmp[0];
      for (int j = 1; j < 4; ++j) {
         f[j] = 0;
         for (int k = 1; k < 4; ++k)
            f[j] += a[k - 1][j - 1] * cmp[k];
      }
      for (int j = 4; j < 10; ++j) {
         f[j] = 0;
         for (int k = 4; k < 10; ++k)
            f[j] += ctf6[k - 4][j - 4] * cmp[k];
      }
   }
}

/* fractional potential -> Cartesian (first 10 components), fphiToCphi_cu1 */
static void or_fphi_to_cphi(const or_pme* p, int n, const double* fphi, int stride, double* cphi)
{
   static const int qi1[6] = {0, 1, 2, 0, 0, 1};
   static const int qi2[6] = {0, 1, 2, 1, 2, 2};
   double a[3][3];
   for (int f = 0; f < 3; ++f)
      for (int c = 0; c < 3; ++c)
         a[f][c] = p->a[f][c];
   double ftc6[6][6];
   for (int i1 = 0; i1 < 3; ++i1) {
      int k = qi1[i1];
      for (int i2 = 0; i2 < 3; ++i2) {
         int ii = qi1[i2];
         ftc6[i2][i1] = a[ii][k] * a[ii][k];
      }
      for (int i2 = 3; i2 < 6; ++i2) {
         int ii = qi1[i2], jj = qi2[i2];
         ftc6[i2][i1] = 2 * a[ii][k] * a[jj][k];
      }
   }
   for (int i1 = 3; i1 < 6; ++i1) {
      int k = qi1[i1], m = qi2[i1];
      for (int i2 = 0; i2 < 3; ++i2) {
         int ii = qi1[i2];
         ftc6[i2][i1] = a[ii][k] * a[ii][m];
      }
      for (int i2 = 3; i2 < 6; ++i2) {
         int ii = qi1[i2], jj = qi2[i2];
         ftc6[i2][i1] = a[ii][k] * a[jj][m] + a[ii][m] * a[jj][k];
      }
   }
   for (int at = 0; at < n; ++at) {
      const double* f = &fphi[(size_t)stride * at];
      double* c = &cphi[10 * at];
      c[0] = f[0];
      for (int j = 1; j < 4; ++j) {
         c[j] = 0;
         for (int k = 1; k < 4; ++k)
            c[j] += a[k - 1][j - 1] * f[k];
      }
      for (int j = 4; j < 10; ++j) {
         c[j] = 0;
         for (int k = 4; k < 10; ++k)
            c[j] += ftc6[k - 4][j - 4] * f[k];
      }
   }
}

/* ------------------------------------------------------------------ */
/* real-space pair terms                                               */

/* pair_dfield_v2 (pair_field.h:127-256), double precision */
static void or_pair_dfield(int ewald, double aewald, double r2, double xr, double yr, double zr, double dscale,
   double pscale, const double* mi, double pdi, double pti, const double* mk, double pdk, double ptk, double fid[3],
   double fip[3], double fkd[3], double fkp[3])
{
   double r = sqrt(r2), invr = 1 / r, rr2 = invr * invr;
   double s3, s5, s7;
   or_thole3(r, pdi, pti, pdk, ptk, &s3, &s5, &s7);
   double bn[4] = {0, 0, 0, 0};
   if (ewald)
      or_ewald_bn(4, bn, r, rr2, aewald);
   double rr3 = invr * rr2, rr5 = 3 * invr * rr2 * rr2, rr7 = 15 * invr * rr2 * rr2 * rr2;
   double ci = mi[0], dix = mi[1], diy = mi[2], diz = mi[3];
   double qixx = mi[4], qiyy = mi[5], qizz = mi[6], qixy = mi[7], qixz = mi[8], qiyz = mi[9];
   double ck = mk[0], dkx = mk[1], dky = mk[2], dkz = mk[3];
   double qkxx = mk[4], qkyy = mk[5], qkzz = mk[6], qkxy = mk[7], qkxz = mk[8], qkyz = mk[9];
   double dir = dix * xr + diy * yr + diz * zr;
   double qix = qixx * xr + qixy * yr + qixz * zr;
   double qiy = qixy * xr + qiyy * yr + qiyz * zr;
   double qiz = qixz * xr + qiyz * yr + qizz * zr;
   double qir = qix * xr + qiy * yr + qiz * zr;
   double dkr = dkx * xr + dky * yr + dkz * zr;
   double qkx = qkxx * xr + qkxy * yr + qkxz * zr;
   double qky = qkxy * xr + qkyy * yr + qkyz * zr;
   double qkz = qkxz * xr + qkyz * yr + qkzz * zr;
   double qkr = qkx * xr + qky * yr + qkz * zr;
   for (int pass = 0; pass < 2; ++pass) {
      double sc = pass == 0 ? dscale : pscale;
      double b1, b2, b3;
      if (ewald) {
         b1 = bn[1] - (1 - sc * s3) * rr3;
         b2 = bn[2] - (1 - sc * s5) * rr5;
         b3 = bn[3] - (1 - sc * s7) * rr7;
      } else {
         b1 = sc * s3 * rr3;
         b2 = sc * s5 * rr5;
         b3 = sc * s7 * rr7;
      }
      double c1 = -(b1 * ck - b2 * dkr + b3 * qkr);
      double ii[3] = {c1 * xr - b1 * dkx + 2 * b2 * qkx, c1 * yr - b1 * dky + 2 * b2 * qky,
         c1 * zr - b1 * dkz + 2 * b2 * qkz};
      double c2 = (b1 * ci + b2 * dir + b3 * qir);
      double kk[3] = {c2 * xr - b1 * dix - 2 * b2 * qix, c2 * yr - b1 * diy - 2 * b2 * qiy,
         c2 * zr - b1 * diz - 2 * b2 * qiz};
      double* fi = pass == 0 ? fid : fip;
      double* fk = pass == 0 ? fkd : fkp;
      for (int d = 0; d < 3; ++d) {
         fi[d] += ii[d];
         fk[d] += kk[d];
      }
   }
}

/* pair_ufield_v2 (pair_field.h:333-420), double precision */
static void or_pair_ufield(int ewald, double aewald, double r2, double xr, double yr, double zr, double uscale,
   const double* uid, const double* uip, double pdi, double pti, const double* ukd, const double* ukp, double pdk,
   double ptk, double fid[3], double fip[3], double fkd[3], double fkp[3])
{
   double r = sqrt(r2), invr = 1 / r, rr2 = invr * invr;
   double s3, s5;
   or_thole3(r, pdi, pti, pdk, ptk, &s3, &s5, NULL);
   double bn[3] = {0, 0, 0};
   double rr3 = invr * rr2, rr5 = 3 * invr * rr2 * rr2;
   double b1, b2;
   if (ewald) {
      or_ewald_bn(3, bn, r, rr2, aewald);
      b1 = bn[1] - (1 - uscale * s3) * rr3;
      b2 = bn[2] - (1 - uscale * s5) * rr5;
   } else {
      b1 = uscale * s3 * rr3;
      b2 = uscale * s5 * rr5;
   }
   const double dr[3] = {xr, yr, zr};
   double c;
   c = b2 * (xr * ukd[0] + yr * ukd[1] + zr * ukd[2]);
   for (int d = 0; d < 3; ++d)
      fid[d] += c * dr[d] - b1 * ukd[d];
   c = b2 * (xr * ukp[0] + yr * ukp[1] + zr * ukp[2]);
   for (int d = 0; d < 3; ++d)
      fip[d] += c * dr[d] - b1 * ukp[d];
   c = b2 * (xr * uid[0] + yr * uid[1] + zr * uid[2]);
   for (int d = 0; d < 3; ++d)
      fkd[d] += c * dr[d] - b1 * uid[d];
   c = b2 * (xr * uip[0] + yr * uip[1] + zr * uip[2]);
   for (int d = 0; d < 3; ++d)
      fkp[d] += c * dr[d] - b1 * uip[d];
}

/* thread-private accumulation of two [n][3] fields */
typedef struct {
   int nt;
   double* buf; /* nt * 6n */
} or_acc;

static void or_acc_init(or_acc* a, int n)
{
   a->nt = or_nthreads();
   a->buf = (double*)calloc((size_t)a->nt * 6 * n, sizeof(double));
}

static void or_acc_reduce(or_acc* a, int n, double* f1, double* f2)
{
   for (int t = 0; t < a->nt; ++t) {
      const double* b = a->buf + (size_t)t * 6 * n;
      for (int i = 0; i < 3 * n; ++i) {
         f1[i] += b[i];
         if (f2)
            f2[i] += b[3 * n + i];
      }
   }
   free(a->buf);
}

static int or_tid(void)
{
#ifdef _OPENMP
   return omp_get_thread_num();
#else
   return 0;
#endif
}

/* ------------------------------------------------------------------ */
/* dfield / ufield (src/amoeba/field.cpp:17-117)                        */

void or_dfield(const or_system* s, double* field, double* fieldp)
{
   const int n = s->n;
   memset(field, 0, sizeof(double) * 3 * n);
   memset(fieldp, 0, sizeof(double) * 3 * n);
   if (s->use_ewald && !s->real_only) {
      or_pme p;
      or_pme_init(s, &p);
      double* fmp = (double*)malloc(sizeof(double) * 10 * n);
      double* fphi = (double*)malloc(sizeof(double) * 20 * n);
      double* cphi = (double*)malloc(sizeof(double) * 10 * n);
      or_cmp_to_fmp(&p, n, s->rpole, fmp);
      or_grid_mpole(s, &p, fmp);
      or_fft3d(p.grid, p.n1, p.n2, p.n3, -1);
      or_pme_conv(s, &p, 0, NULL);
      or_fft3d(p.grid, p.n1, p.n2, p.n3, +1);
      or_fphi(s, &p, 0, 20, fphi, 20);
      or_fphi_to_cphi(&p, n, fphi, 20, cphi);
      const double term = s->aewald * s->aewald * s->aewald * 4 / 3 / OR_SQRTPI;
      for (int i = 0; i < n; ++i)
         for (int d = 0; d < 3; ++d) {
            field[3 * i + d] = -cphi[10 * i + 1 + d] + term * s->rpole[10 * i + 1 + d];
            fieldp[3 * i + d] = field[3 * i + d];
         }
      free(fmp);
      free(fphi);
      free(cphi);
      or_pme_free(&p);
   }
   or_pairs pl;
   or_build_pairs(s, s->cutoff, &pl);
   or_excl ex;
   or_excl_build(s, &ex);
   or_acc acc;
   or_acc_init(&acc, n);
#pragma omp parallel for schedule(dynamic, 256)
   for (int j = 0; j < pl.npair; ++j) {
      double* fd = acc.buf + (size_t)or_tid() * 6 * n;
      double* fp = fd + 3 * n;
      int i = pl.ik[2 * j], k = pl.ik[2 * j + 1];
      double xr = s->x[k] - s->x[i], yr = s->y[k] - s->y[i], zr = s->z[k] - s->z[i];
      or_image(s, &xr, &yr, &zr);
      double r2 = xr * xr + yr * yr + zr * zr;
      double sc[4];
      or_excl_get(s, &ex, i, k, sc);
      const double pga = or_pair_gamma(s, i, k);
      or_pair_dfield(s->use_ewald, s->aewald, r2, xr, yr, zr, sc[1], sc[2], &s->rpole[10 * i], s->pdamp[i],
         pga, &s->rpole[10 * k], s->pdamp[k], pga, &fd[3 * i], &fp[3 * i], &fd[3 * k], &fp[3 * k]);
   }
   or_acc_reduce(&acc, n, field, fieldp);
   or_excl_free(&ex);
   or_pairs_free(&pl);
   /* external field on both sets (extfieldModifyDField, src/cu/amoeba/empole.cu:139-159) */
   for (int i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) {
         field[3 * i + d] += s->exfld[d];
         fieldp[3 * i + d] += s->exfld[d];
      }
}

/* cached pair list and PME state for repeated ufield calls */
typedef struct {
   or_pairs pl;
   or_excl ex;
   or_pme pme;
   int have_pme;
} or_ucache;

static void or_ucache_init(const or_system* s, or_ucache* c)
{
   or_build_pairs(s, s->cutoff, &c->pl);
   or_excl_build(s, &c->ex);
   c->have_pme = s->use_ewald;
   if (c->have_pme)
      or_pme_init(s, &c->pme);
}

static void or_ucache_free(or_ucache* c)
{
   or_pairs_free(&c->pl);
   or_excl_free(&c->ex);
   if (c->have_pme)
      or_pme_free(&c->pme);
}

static void or_ufield_c(const or_system* s, or_ucache* c, const double* uind, const double* uinp, double* field,
   double* fieldp)
{
   const int n = s->n;
   memset(field, 0, sizeof(double) * 3 * n);
   memset(fieldp, 0, sizeof(double) * 3 * n);
   if (s->use_ewald && !s->real_only) {
      or_pme* p = &c->pme;
      double* fuind = (double*)malloc(sizeof(double) * 3 * n);
      double* fuinp = (double*)malloc(sizeof(double) * 3 * n);
      double* phi1 = (double*)malloc(sizeof(double) * 10 * n);
      double* phi2 = (double*)malloc(sizeof(double) * 10 * n);
      for (int i = 0; i < n; ++i)
         for (int f = 0; f < 3; ++f) {
            fuind[3 * i + f] = 0;
            fuinp[3 * i + f] = 0;
            for (int k = 0; k < 3; ++k) {
               fuind[3 * i + f] += p->a[f][k] * uind[3 * i + k];
               fuinp[3 * i + f] += p->a[f][k] * uinp[3 * i + k];
            }
         }
      or_grid_uind(s, p, fuind, fuinp);
      or_fft3d(p->grid, p->n1, p->n2, p->n3, -1);
      or_pme_conv(s, p, 0, NULL);
      or_fft3d(p->grid, p->n1, p->n2, p->n3, +1);
      or_fphi(s, p, 0, 10, phi1, 10);
      or_fphi(s, p, 1, 10, phi2, 10);
      const double term = s->aewald * s->aewald * s->aewald * 4 / 3 / OR_SQRTPI;
      for (int i = 0; i < n; ++i)
         for (int cc = 0; cc < 3; ++cc) {
            double df1 = 0, df2 = 0;
            for (int f = 0; f < 3; ++f) {
               df1 += p->a[f][cc] * phi1[10 * i + 1 + f];
               df2 += p->a[f][cc] * phi2[10 * i + 1 + f];
            }
            field[3 * i + cc] = term * uind[3 * i + cc] - df1;
            fieldp[3 * i + cc] = term * uinp[3 * i + cc] - df2;
         }
      free(fuind);
      free(fuinp);
      free(phi1);
      free(phi2);
   }
   or_acc acc;
   or_acc_init(&acc, n);
   const or_pairs* pl = &c->pl;
#pragma omp parallel for schedule(dynamic, 256)
   for (int j = 0; j < pl->npair; ++j) {
      double* fd = acc.buf + (size_t)or_tid() * 6 * n;
      double* fp = fd + 3 * n;
      int i = pl->ik[2 * j], k = pl->ik[2 * j + 1];
      double xr = s->x[k] - s->x[i], yr = s->y[k] - s->y[i], zr = s->z[k] - s->z[i];
      or_image(s, &xr, &yr, &zr);
      double r2 = xr * xr + yr * yr + zr * zr;
      double sc[4];
      or_excl_get(s, &c->ex, i, k, sc);
      const double pga = or_pair_gamma(s, i, k);
      or_pair_ufield(s->use_ewald, s->aewald, r2, xr, yr, zr, sc[3], &uind[3 * i], &uinp[3 * i], s->pdamp[i],
         pga, &uind[3 * k], &uinp[3 * k], s->pdamp[k], pga, &fd[3 * i], &fp[3 * i], &fd[3 * k], &fp[3 * k]);
   }
   or_acc_reduce(&acc, n, field, fieldp);
}

void or_ufield(const or_system* s, const double* uind, const double* uinp, double* field, double* fieldp)
{
   or_ucache c;
   or_ucache_init(s, &c);
   or_ufield_c(s, &c, uind, uinp, field, fieldp);
   or_ucache_free(&c);
}

/* ------------------------------------------------------------------ */
/* preconditioners                                                      */

static void or_sparse_precond(const or_system* s, const or_pairs* pl, const or_excl* ex, double udiag,
   const double* rsd, const double* rsdp, double* zrsd, double* zrsdp)
{
   const int n = s->n;
   for (int i = 0; i < n; ++i) {
      double poli = udiag * s->polarity[i];
      for (int d = 0; d < 3; ++d) {
         zrsd[3 * i + d] = poli * rsd[3 * i + d];
         zrsdp[3 * i + d] = poli * rsdp[3 * i + d];
      }
   }
   or_acc acc;
   or_acc_init(&acc, n);
#pragma omp parallel for schedule(dynamic, 256)
   for (int j = 0; j < pl->npair; ++j) {
      double* fd = acc.buf + (size_t)or_tid() * 6 * n;
      double* fp = fd + 3 * n;
      int i = pl->ik[2 * j], k = pl->ik[2 * j + 1];
      double xr = s->x[k] - s->x[i], yr = s->y[k] - s->y[i], zr = s->z[k] - s->z[i];
      or_image(s, &xr, &yr, &zr);
      double r2 = xr * xr + yr * yr + zr * zr;
      double r = sqrt(r2);
      double sc[4];
      or_excl_get(s, ex, i, k, sc);
      double s3, s5;
      const double pga = or_pair_gamma(s, i, k);
      or_thole3(r, s->pdamp[i], pga, s->pdamp[k], pga, &s3, &s5, NULL);
      s3 *= sc[3];
      s5 *= sc[3];
      double polik = s->polarity[i] * s->polarity[k];
      double rr3 = s3 * polik / (r * r2);
      double rr5 = 3 * s5 * polik / (r * r2 * r2);
      const double dr[3] = {xr, yr, zr};
      const double *ukd = &rsd[3 * k], *ukp = &rsdp[3 * k], *uid = &rsd[3 * i], *uip = &rsdp[3 * i];
      double c;
      c = rr5 * (xr * ukd[0] + yr * ukd[1] + zr * ukd[2]);
      for (int d = 0; d < 3; ++d)
         fd[3 * i + d] += c * dr[d] - rr3 * ukd[d];
      c = rr5 * (xr * ukp[0] + yr * ukp[1] + zr * ukp[2]);
      for (int d = 0; d < 3; ++d)
         fp[3 * i + d] += c * dr[d] - rr3 * ukp[d];
      c = rr5 * (xr * uid[0] + yr * uid[1] + zr * uid[2]);
      for (int d = 0; d < 3; ++d)
         fd[3 * k + d] += c * dr[d] - rr3 * uid[d];
      c = rr5 * (xr * uip[0] + yr * uip[1] + zr * uip[2]);
      for (int d = 0; d < 3; ++d)
         fp[3 * k + d] += c * dr[d] - rr3 * uip[d];
   }
   or_acc_reduce(&acc, n, zrsd, zrsdp);
}

void or_sparse_precond_apply(const or_system* s, double cutoff, double udiag, const double* rsd, const double* rsdp,
   double* zrsd, double* zrsdp)
{
   or_pairs pl;
   or_build_pairs(s, cutoff, &pl);
   or_excl ex;
   or_excl_build(s, &ex);
   or_sparse_precond(s, &pl, &ex, udiag, rsd, rsdp, zrsd, zrsdp);
   or_excl_free(&ex);
   or_pairs_free(&pl);
}

static double or_dot(int n3, const double* a, const double* b)
{
   double s = 0;
   for (int i = 0; i < n3; ++i)
      s += a[i] * b[i];
   return s;
}

/* ------------------------------------------------------------------ */
/* PCG (src/cu/amoeba/pcg.cu:14-185)                                    */

/* uind/uinp: in = caller guess when opts->guess == 2, out = converged dipoles.
 * udir/udirp (optional) receive alpha*E.  Returns the iteration count; *eps_out
 * receives the final RMS residual in Debye. */
int or_induce(const or_system* s, const or_induce_opts* o, double* uind, double* uinp, double* udir_out,
   double* udirp_out, double* eps_out)
{
   const int n = s->n, n3 = 3 * n;
   double* field = (double*)malloc(sizeof(double) * n3);
   double* fieldp = (double*)malloc(sizeof(double) * n3);
   double* udir = (double*)malloc(sizeof(double) * n3);
   double* udirp = (double*)malloc(sizeof(double) * n3);
   double* rsd = (double*)malloc(sizeof(double) * n3);
   double* rsdp = (double*)malloc(sizeof(double) * n3);
   double* zrsd = (double*)malloc(sizeof(double) * n3);
   double* zrsdp = (double*)malloc(sizeof(double) * n3);
   double* conj = (double*)malloc(sizeof(double) * n3);
   double* conjp = (double*)malloc(sizeof(double) * n3);
   double* vec = (double*)malloc(sizeof(double) * n3);
   double* vecp = (double*)malloc(sizeof(double) * n3);
   double* pinv = (double*)malloc(sizeof(double) * n);
   for (int i = 0; i < n; ++i)
      pinv[i] = 1.0 / fmax(s->polarity[i], 1.0e-16);

   or_ucache uc;
   or_ucache_init(s, &uc);
   or_pairs ppl = {0, NULL};
   if (o->pcgprec)
      or_build_pairs(s, o->precond_cutoff, &ppl);

   or_dfield(s, field, fieldp);
   for (int i = 0; i < n; ++i)
      for (int d = 0; d < 3; ++d) {
         udir[3 * i + d] = s->polarity[i] * field[3 * i + d];
         udirp[3 * i + d] = s->polarity[i] * fieldp[3 * i + d];
      }
   if (udir_out)
      memcpy(udir_out, udir, sizeof(double) * n3);
   if (udirp_out)
      memcpy(udirp_out, udirp, sizeof(double) * n3);

   if (o->guess == 2) {
      or_ufield_c(s, &uc, uind, uinp, field, fieldp);
      for (int i = 0; i < n; ++i)
         for (int d = 0; d < 3; ++d) {
            rsd[3 * i + d] = (udir[3 * i + d] - uind[3 * i + d]) * pinv[i] + field[3 * i + d];
            rsdp[3 * i + d] = (udirp[3 * i + d] - uinp[3 * i + d]) * pinv[i] + fieldp[3 * i + d];
         }
   } else if (o->guess == 1) {
      memcpy(uind, udir, sizeof(double) * n3);
      memcpy(uinp, udirp, sizeof(double) * n3);
      or_ufield_c(s, &uc, uind, uinp, rsd, rsdp);
   } else {
      memset(uind, 0, sizeof(double) * n3);
      memset(uinp, 0, sizeof(double) * n3);
      memcpy(rsd, field, sizeof(double) * n3);
      memcpy(rsdp, fieldp, sizeof(double) * n3);
   }
   for (int i = 0; i < n; ++i)
      if (s->polarity[i] == 0)
         for (int d = 0; d < 3; ++d)
            rsd[3 * i + d] = rsdp[3 * i + d] = 0;

#define OR_PRECOND()                                                                                                   \
   do {                                                                                                                \
      if (o->pcgprec)                                                                                                  \
         or_sparse_precond(s, &ppl, &uc.ex, o->udiag, rsd, rsdp, zrsd, zrsdp);                                         \
      else                                                                                                             \
         for (int i = 0; i < n; ++i)                                                                                   \
            for (int d = 0; d < 3; ++d) {                                                                              \
               zrsd[3 * i + d] = s->polarity[i] * rsd[3 * i + d];                                                      \
               zrsdp[3 * i + d] = s->polarity[i] * rsdp[3 * i + d];                                                    \
            }                                                                                                          \
   } while (0)

   OR_PRECOND();
   memcpy(conj, zrsd, sizeof(double) * n3);
   memcpy(conjp, zrsdp, sizeof(double) * n3);
   double sum = or_dot(n3, rsd, zrsd), sump = or_dot(n3, rsdp, zrsdp);

   const int miniter = n < 3 ? n : 3;
   int iter = 0, done = 0;
   double eps = 100;
   while (!done) {
      ++iter;
      or_ufield_c(s, &uc, conj, conjp, field, fieldp);
      for (int i = 0; i < n; ++i)
         for (int d = 0; d < 3; ++d) {
            vec[3 * i + d] = pinv[i] * conj[3 * i + d] - field[3 * i + d];
            vecp[3 * i + d] = pinv[i] * conjp[3 * i + d] - fieldp[3 * i + d];
         }
      double a = or_dot(n3, conj, vec), ap = or_dot(n3, conjp, vecp);
      a = (a == 0) ? 0 : sum / a;
      ap = (ap == 0) ? 0 : sump / ap;
      for (int i = 0; i < n; ++i) {
         for (int d = 0; d < 3; ++d) {
            uind[3 * i + d] += a * conj[3 * i + d];
            uinp[3 * i + d] += ap * conjp[3 * i + d];
            rsd[3 * i + d] -= a * vec[3 * i + d];
            rsdp[3 * i + d] -= ap * vecp[3 * i + d];
         }
         if (s->polarity[i] == 0)
            for (int d = 0; d < 3; ++d)
               rsd[3 * i + d] = rsdp[3 * i + d] = 0;
      }
      OR_PRECOND();
      double sum1 = or_dot(n3, rsd, zrsd), sump1 = or_dot(n3, rsdp, zrsdp);
      double b = (sum == 0) ? 0 : sum1 / sum, bp = (sump == 0) ? 0 : sump1 / sump;
      for (int i = 0; i < n3; ++i) {
         conj[i] = zrsd[i] + b * conj[i];
         conjp[i] = zrsdp[i] + bp * conjp[i];
      }
      sum = sum1;
      sump = sump1;
      double ed = or_dot(n3, rsd, rsd), ep = or_dot(n3, rsdp, rsdp);
      eps = o->debye * sqrt(fmax(ed, ep) / n);
      if (eps < o->poleps)
         done = 1;
      if (iter < miniter)
         done = 0;
      if (iter >= o->politer)
         done = 1;
      if (done)
         for (int i = 0; i < n; ++i) {
            double term = o->pcgpeek * s->polarity[i];
            for (int d = 0; d < 3; ++d) {
               uind[3 * i + d] += term * rsd[3 * i + d];
               uinp[3 * i + d] += term * rsdp[3 * i + d];
            }
         }
   }
#undef OR_PRECOND
   if (eps_out)
      *eps_out = eps;
   or_ucache_free(&uc);
   if (o->pcgprec)
      or_pairs_free(&ppl);
   free(field);
   free(fieldp);
   free(udir);
   free(udirp);
   free(rsd);
   free(rsdp);
   free(zrsd);
   free(zrsdp);
   free(conj);
   free(conjp);
   free(vec);
   free(vecp);
   free(pinv);
   return iter;
}

/* ASPC extrapolation weights (Kolafa, J. Comput. Chem. 25, 335 (2004)); the
 * reference tabulates the same 16 values in src/cu/upredict.cu:40-55. */
static const double or_aspc[16] = {62. / 17., -310. / 51., 2170. / 323., -2329. / 400., 1701. / 409., -806. / 323.,
   1024. / 809., -479. / 883., 257. / 1316., -434. / 7429., 191. / 13375., -62. / 22287., 3. / 7217.,
   -3. / 67015., 2. / 646323., -1. / 9694845.};

/* hist[16][n3] ring buffer, nualt = saves so far; slot s gets aspc[(nualt-1-s) mod 16] */
void or_aspc_sum(int n3, int nualt, const double* hist, double* u)
{
   for (int i = 0; i < n3; ++i) {
      double acc = 0;
      for (int s = 0; s < 16; ++s)
         acc += or_aspc[((nualt - 1 - s) % 16 + 16) % 16] * hist[(size_t)s * n3 + i];
      u[i] = acc;
   }
}

/* Gear 6-point extrapolation, the binomial weights of the fifth difference
 * (exact for a quintic history); the reference's table is in
 * src/cu/upredict.cu:141-146 and its ring of 6 in src/amoeba/epolar.cpp:461-468.
 * hist[6][n3], slot s gets gear[(nualt-1-s) mod 6]. */
static const double or_gear[6] = {6., -15., 20., -15., 6., -1.};

void or_gear_sum(int n3, int nualt, const double* hist, double* u)
{
   for (int i = 0; i < n3; ++i) {
      double acc = 0;
      for (int s = 0; s < 6; ++s)
         acc += or_gear[((nualt - 1 - s) % 6 + 6) % 6] * hist[(size_t)s * n3 + i];
      u[i] = acc;
   }
}

/* exported wrappers for tests: PME pieces */
void or_bsplgen_export(double w, int order, int level, double* theta) { or_bsplgen(w, order, level, theta); }

double or_pme_energy_uind_check(const or_system* s, const double* fuind, const double* fuinp, double* grid_out)
{
   or_pme p;
   or_pme_init(s, &p);
   or_grid_uind(s, &p, fuind, fuinp);
   size_t ng = (size_t)p.n1 * p.n2 * p.n3;
   if (grid_out)
      for (size_t j = 0; j < ng; ++j) {
         grid_out[2 * j] = creal(p.grid[j]);
         grid_out[2 * j + 1] = cimag(p.grid[j]);
      }
   or_pme_free(&p);
   return 0;
}

/* ------------------------------------------------------------------ */
/* energies consuming the multipoles and converged dipoles              */

/* pair_mpole energy (include/seq/pair_mpole.h:62-152): bn already scaled */
static double or_mpole_pair_e(const double* bn, double xr, double yr, double zr, const double* mi, const double* mk)
{
   double ci = mi[0], dix = mi[1], diy = mi[2], diz = mi[3];
   double qixx = mi[4], qiyy = mi[5], qizz = mi[6], qixy = mi[7], qixz = mi[8], qiyz = mi[9];
   double ck = mk[0], dkx = mk[1], dky = mk[2], dkz = mk[3];
   double qkxx = mk[4], qkyy = mk[5], qkzz = mk[6], qkxy = mk[7], qkxz = mk[8], qkyz = mk[9];
   double dir = dix * xr + diy * yr + diz * zr;
   double qix = qixx * xr + qixy * yr + qixz * zr;
   double qiy = qixy * xr + qiyy * yr + qiyz * zr;
   double qiz = qixz * xr + qiyz * yr + qizz * zr;
   double qir = qix * xr + qiy * yr + qiz * zr;
   double dkr = dkx * xr + dky * yr + dkz * zr;
   double qkx = qkxx * xr + qkxy * yr + qkxz * zr;
   double qky = qkxy * xr + qkyy * yr + qkyz * zr;
   double qkz = qkxz * xr + qkyz * yr + qkzz * zr;
   double qkr = qkx * xr + qky * yr + qkz * zr;
   double dik = dix * dkx + diy * dky + diz * dkz;
   double qik = qix * qkx + qiy * qky + qiz * qkz;
   double diqk = dix * qkx + diy * qky + diz * qkz;
   double dkqi = dkx * qix + dky * qiy + dkz * qiz;
   double qiqk = 2 * (qixy * qkxy + qixz * qkxz + qiyz * qkyz) + qixx * qkxx + qiyy * qkyy + qizz * qkzz;
   double term1 = ci * ck;
   double term2 = ck * dir - ci * dkr + dik;
   double term3 = ci * qkr + ck * qir - dir * dkr + 2 * (dkqi - diqk + qiqk);
   double term4 = dir * qkr - dkr * qir - 4 * qik;
   double term5 = qir * qkr;
   return term1 * bn[0] + term2 * bn[1] + term3 * bn[2] + term4 * bn[3] + term5 * bn[4];
}

/* Permanent-multipole energy split into real, reciprocal and self parts
 * (src/amoeba/empole.cpp:81-138; real space empole_cu1.cc with the
 * exclusion correction (m - 1) x bare pair, empole_cu1.cc:110; recip
 * 0.5 f sum fmp.fphi, src/cu/hippo/empole.cu:202-335; self
 * include/seq/emselfamoeba.h:7-37).  Non-Ewald: parts[0] only. */
double or_empole_energy(const or_system* s, double* parts)
{
   const int n = s->n;
   const double f = s->electric;
   double ereal = 0, erecip = 0, eself = 0;
   or_pairs pl;
   or_build_pairs(s, s->cutoff, &pl);
   or_excl ex;
   or_excl_build(s, &ex);
#pragma omp parallel for reduction(+ : ereal) schedule(dynamic, 256)
   for (int j = 0; j < pl.npair; ++j) {
      int i = pl.ik[2 * j], k = pl.ik[2 * j + 1];
      double xr = s->x[k] - s->x[i], yr = s->y[k] - s->y[i], zr = s->z[k] - s->z[i];
      or_image(s, &xr, &yr, &zr);
      double r2 = xr * xr + yr * yr + zr * zr;
      double r = sqrt(r2), rr2 = 1 / r2;
      double sc[4];
      or_excl_get(s, &ex, i, k, sc);
      double bare[5];
      bare[0] = f / r;
      bare[1] = bare[0] * rr2;
      bare[2] = 3 * bare[1] * rr2;
      bare[3] = 5 * bare[2] * rr2;
      bare[4] = 7 * bare[3] * rr2;
      double e;
      if (s->use_ewald) {
         double bn[5];
         or_ewald_bn(5, bn, r, rr2, s->aewald);
         for (int q = 0; q < 5; ++q)
            bn[q] *= f;
         e = or_mpole_pair_e(bn, xr, yr, zr, &s->rpole[10 * i], &s->rpole[10 * k]);
         if (sc[0] != 1)
            e += (sc[0] - 1) * or_mpole_pair_e(bare, xr, yr, zr, &s->rpole[10 * i], &s->rpole[10 * k]);
      } else {
         e = sc[0] * or_mpole_pair_e(bare, xr, yr, zr, &s->rpole[10 * i], &s->rpole[10 * k]);
      }
      ereal += e;
   }
   or_excl_free(&ex);
   or_pairs_free(&pl);
   if (s->use_ewald) {
      or_pme p;
      or_pme_init(s, &p);
      double* fmp = (double*)malloc(sizeof(double) * 10 * n);
      double* fphi = (double*)malloc(sizeof(double) * 20 * n);
      or_cmp_to_fmp(&p, n, s->rpole, fmp);
      or_grid_mpole(s, &p, fmp);
      or_fft3d(p.grid, p.n1, p.n2, p.n3, -1);
      or_pme_conv(s, &p, 0, NULL);
      or_fft3d(p.grid, p.n1, p.n2, p.n3, +1);
      or_fphi(s, &p, 0, 10, fphi, 20);
      for (int i = 0; i < n; ++i)
         for (int c = 0; c < 10; ++c)
            erecip += 0.5 * f * fmp[10 * i + c] * fphi[20 * i + c];
      free(fmp);
      free(fphi);
      or_pme_free(&p);
      const double a = s->aewald, a2 = 2 * a * a;
      const double fterm = -f * a / OR_SQRTPI;
      for (int i = 0; i < n; ++i) {
         const double* m = &s->rpole[10 * i];
         double cii = m[0] * m[0];
         double dii = m[1] * m[1] + m[2] * m[2] + m[3] * m[3];
         double qii = 2 * (m[7] * m[7] + m[8] * m[8] + m[9] * m[9]) + m[4] * m[4] + m[5] * m[5] + m[6] * m[6];
         eself += fterm * (cii + a2 * (dii / 3 + 2 * a2 * qii * 0.2));
      }
   }
   /* permanent multipoles in the external field, -f (q r.E + d.E) per atom
    * with unwrapped coordinates (exfieldDipole_cu1, src/cu/amoeba/empole.cu:79-130);
    * counted with the one-body self part */
   for (int i = 0; i < n; ++i) {
      const double* m = &s->rpole[10 * i];
      const double* E = s->exfld;
      eself -= f * (m[0] * (s->x[i] * E[0] + s->y[i] * E[1] + s->z[i] * E[2]) + m[1] * E[0] + m[2] * E[1] +
                      m[3] * E[2]);
   }
   if (parts) {
      parts[0] = ereal;
      parts[1] = erecip;
      parts[2] = eself;
   }
   return ereal + erecip + eself;
}

/* Polarization energy by the dot product -1/2 f sum_i u_d,i . E_p,i with
 * E_p = udirp / alpha (src/cu/amoeba/epolar.cu:14-30). */
double or_epolar_energy_dot(const or_system* s, const double* uind, const double* udirp)
{
   double e = 0;
   for (int i = 0; i < s->n; ++i) {
      double pinv = 1.0 / fmax(s->polarity[i], 1.0e-16);
      e += pinv * (uind[3 * i] * udirp[3 * i] + uind[3 * i + 1] * udirp[3 * i + 1] + uind[3 * i + 2] * udirp[3 * i + 2]);
   }
   return -0.5 * s->electric * e;
}
