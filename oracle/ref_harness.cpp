// Reference-code harness: the reference's own per-pair and per-site
// arithmetic (Tinker9 include/seq/*.h, include/ff/image.h), compiled from
// its source tree in double precision (TINKER_DOUBLE_PRECISION) by
// oracle/build_ref.py into oracle/_ref/libt9ref.so.
//
// TEST INFRASTRUCTURE ONLY.  The loops are written here and follow the
// structure of the reference's host (OpenACC) path, whose pragmas g++
// ignores: a pass over every pair within the cutoff at scale 1, then a pass
// over the scaled pairs with (scale - 1) and the non-Ewald kernel
// (src/acc/amoeba/fieldewald.cpp:33-200, 260-400;
// src/acc/amoeba/empoleewald.cpp:20-190).  The per-pair functions are the
// reference's: pair_dfield / pair_ufield (include/seq/pair_field.h:9-124,
// 259-330), pair_mpole (include/seq/pair_mpole.h:63-235), with damp_thole3 /
// damp_thole2 / damp_ewald and the Hastings-free double erfc of
// include/seq/damp.h and include/math/libfunc.h; chkpoleAtomI / rotpoleAtomI
// (include/seq/rotpole.h:9-200); bsplgen (include/seq/bsplgen.h:27-116);
// image2General (include/ff/image.h:165-170).  The oracle (t9_oracle.c) is
// compared with these on the same inputs by tests/test_oracle_reference_build.py.
#include "ff/amoeba/mpole.h"
#include "ff/box.h"
#include "ff/image.h"
#include "seq/bsplgen.h"
#include "seq/pair_field.h"
#include "seq/pair_mpole.h"
#include "seq/rotpole.h"

#include <vector>

using namespace tinker;

extern "C" {

typedef struct {
   int n;
   const double* x;
   const double* y;
   const double* z;
   const double* rpole;      // [n][10] global frame, MPL_PME order
   const double* pdamp;      // [n]
   const double* thole;      // [n]
   int nexcl;                // scaled pairs, i < k
   const int* excl_ik;       // [nexcl][2]
   const double* excl_scale; // [nexcl][4]: m, d, p, u
   int periodic;             // orthorhombic box when 1
   double box[3];
   int use_ewald;
   double aewald;
   double cutoff;
   double electric;
} ref_system;

}  // extern "C"

namespace {

struct Image
{
   BoxShape sh;
   real3 l1, l2, l3, ra, rb, rc;
};

Image make_image(const ref_system* s)
{
   Image im;
   im.sh = s->periodic ? BoxShape::ORTHO : BoxShape::UNBOUND;
   const double a = s->periodic ? s->box[0] : 1, b = s->periodic ? s->box[1] : 1, c = s->periodic ? s->box[2] : 1;
   // lvec rows and reciprocal rows of an orthorhombic box (src/box.cpp)
   im.l1 = make_real3(a, 0, 0);
   im.l2 = make_real3(0, b, 0);
   im.l3 = make_real3(0, 0, c);
   im.ra = make_real3(1 / a, 0, 0);
   im.rb = make_real3(0, 1 / b, 0);
   im.rc = make_real3(0, 0, 1 / c);
   return im;
}

// r2 and the minimum-image vector from i to k
real pair_r(const ref_system* s, const Image& im, int i, int k, real& xr, real& yr, real& zr)
{
   xr = s->x[k] - s->x[i];
   yr = s->y[k] - s->y[i];
   zr = s->z[k] - s->z[i];
   return image2General(xr, yr, zr, im.sh, im.l1, im.l2, im.l3, im.ra, im.rb, im.rc);
}

template <class F>
void each_pair(const ref_system* s, F&& f)
{
   for (int i = 0; i < s->n; ++i)
      for (int k = i + 1; k < s->n; ++k)
         f(i, k);
}

#define RP(i) s->rpole[10 * (i) + 0], s->rpole[10 * (i) + 1], s->rpole[10 * (i) + 2], s->rpole[10 * (i) + 3], \
   s->rpole[10 * (i) + 4], s->rpole[10 * (i) + 7], s->rpole[10 * (i) + 8], s->rpole[10 * (i) + 5],              \
   s->rpole[10 * (i) + 9], s->rpole[10 * (i) + 6]

template <class ETYP>
void dfield_pair(const ref_system* s, int i, int k, real xr, real yr, real zr, real r2, real dsc, real psc,
   double* f, double* fp)
{
   real3 fid = make_real3(0, 0, 0), fip = make_real3(0, 0, 0), fkd = make_real3(0, 0, 0), fkp = make_real3(0, 0, 0);
   pair_dfield<ETYP>(r2, xr, yr, zr, dsc, psc, RP(i), s->pdamp[i], s->thole[i], RP(k), s->pdamp[k], s->thole[k],
      s->aewald, fid, fip, fkd, fkp);
   f[3 * i] += fid.x, f[3 * i + 1] += fid.y, f[3 * i + 2] += fid.z;
   fp[3 * i] += fip.x, fp[3 * i + 1] += fip.y, fp[3 * i + 2] += fip.z;
   f[3 * k] += fkd.x, f[3 * k + 1] += fkd.y, f[3 * k + 2] += fkd.z;
   fp[3 * k] += fkp.x, fp[3 * k + 1] += fkp.y, fp[3 * k + 2] += fkp.z;
}

template <class ETYP>
void ufield_pair(const ref_system* s, int i, int k, real xr, real yr, real zr, real r2, real usc, const double* ud,
   const double* up, double* f, double* fp)
{
   real3 fid = make_real3(0, 0, 0), fip = make_real3(0, 0, 0), fkd = make_real3(0, 0, 0), fkp = make_real3(0, 0, 0);
   pair_ufield<ETYP>(r2, xr, yr, zr, usc, ud[3 * i], ud[3 * i + 1], ud[3 * i + 2], up[3 * i], up[3 * i + 1],
      up[3 * i + 2], s->pdamp[i], s->thole[i], ud[3 * k], ud[3 * k + 1], ud[3 * k + 2], up[3 * k], up[3 * k + 1],
      up[3 * k + 2], s->pdamp[k], s->thole[k], s->aewald, fid, fip, fkd, fkp);
   f[3 * i] += fid.x, f[3 * i + 1] += fid.y, f[3 * i + 2] += fid.z;
   fp[3 * i] += fip.x, fp[3 * i + 1] += fip.y, fp[3 * i + 2] += fip.z;
   f[3 * k] += fkd.x, f[3 * k + 1] += fkd.y, f[3 * k + 2] += fkd.z;
   fp[3 * k] += fkp.x, fp[3 * k + 1] += fkp.y, fp[3 * k + 2] += fkp.z;
}

}  // namespace

extern "C" {

// local -> global multipoles with the chirality check; pole_local is
// copied (chkpoleAtomI flips it in place)
void ref_rotpole(int n, const int* frames, const double* pole_local, const double* x, const double* y,
   const double* z, double* rpole)
{
   std::vector<LocalFrame> fr(n);
   for (int i = 0; i < n; ++i)
      fr[i] = LocalFrame{frames[4 * i], frames[4 * i + 1], frames[4 * i + 2], frames[4 * i + 3]};
   std::vector<double> pole(pole_local, pole_local + 10 * (size_t)n);
   auto* p = reinterpret_cast<real(*)[MPL_TOTAL]>(pole.data());
   auto* rp = reinterpret_cast<real(*)[MPL_TOTAL]>(rpole);
   for (int i = 0; i < n; ++i) {
      chkpoleAtomI(i, p, fr.data(), x, y, z);
      rotpoleAtomI(i, rp, p, fr.data(), x, y, z);
   }
}

// real-space (use_ewald) or damped-Coulomb permanent field, d and p sets
void ref_dfield_real(const ref_system* s, double* field, double* fieldp)
{
   const Image im = make_image(s);
   const real off2 = s->cutoff * s->cutoff;
   for (int j = 0; j < 3 * s->n; ++j)
      field[j] = fieldp[j] = 0;
   each_pair(s, [&](int i, int k) {
      real xr, yr, zr;
      const real r2 = pair_r(s, im, i, k, xr, yr, zr);
      if (r2 > off2)
         return;
      if (s->use_ewald)
         dfield_pair<EWALD>(s, i, k, xr, yr, zr, r2, 1, 1, field, fieldp);
      else
         dfield_pair<NON_EWALD>(s, i, k, xr, yr, zr, r2, 1, 1, field, fieldp);
   });
   for (int e = 0; e < s->nexcl; ++e) {
      const int i = s->excl_ik[2 * e], k = s->excl_ik[2 * e + 1];
      const real dsc = s->excl_scale[4 * e + 1] - 1, psc = s->excl_scale[4 * e + 2] - 1;
      real xr, yr, zr;
      const real r2 = pair_r(s, im, i, k, xr, yr, zr);
      if (r2 <= off2)
         dfield_pair<NON_EWALD>(s, i, k, xr, yr, zr, r2, dsc, psc, field, fieldp);
   }
}

// real-space (use_ewald) or damped-Coulomb mutual field -T u
void ref_ufield_real(const ref_system* s, const double* uind, const double* uinp, double* field, double* fieldp)
{
   const Image im = make_image(s);
   const real off2 = s->cutoff * s->cutoff;
   for (int j = 0; j < 3 * s->n; ++j)
      field[j] = fieldp[j] = 0;
   each_pair(s, [&](int i, int k) {
      real xr, yr, zr;
      const real r2 = pair_r(s, im, i, k, xr, yr, zr);
      if (r2 > off2)
         return;
      if (s->use_ewald)
         ufield_pair<EWALD>(s, i, k, xr, yr, zr, r2, 1, uind, uinp, field, fieldp);
      else
         ufield_pair<NON_EWALD>(s, i, k, xr, yr, zr, r2, 1, uind, uinp, field, fieldp);
   });
   for (int e = 0; e < s->nexcl; ++e) {
      const int i = s->excl_ik[2 * e], k = s->excl_ik[2 * e + 1];
      const real usc = s->excl_scale[4 * e + 3] - 1;
      if (usc == 0)
         continue;
      real xr, yr, zr;
      const real r2 = pair_r(s, im, i, k, xr, yr, zr);
      if (r2 <= off2)
         ufield_pair<NON_EWALD>(s, i, k, xr, yr, zr, r2, usc, uind, uinp, field, fieldp);
   }
}

// real-space (use_ewald) or plain multipole energy, kcal/mol
double ref_empole_real(const ref_system* s)
{
   const Image im = make_image(s);
   const real off2 = s->cutoff * s->cutoff;
   const real f = s->electric;
   double etot = 0;
   each_pair(s, [&](int i, int k) {
      real xr, yr, zr;
      const real r2 = pair_r(s, im, i, k, xr, yr, zr);
      if (r2 > off2)
         return;
      real e = 0;
      PairMPoleGrad pg;
      zero(pg);
      if (s->use_ewald)
         pair_mpole<true, false, EWALD>(r2, xr, yr, zr, 1, RP(i), RP(k), f, s->aewald, e, pg);
      else
         pair_mpole<true, false, NON_EWALD>(r2, xr, yr, zr, 1, RP(i), RP(k), f, 0, e, pg);
      etot += e;
   });
   for (int j = 0; j < s->nexcl; ++j) {
      const int i = s->excl_ik[2 * j], k = s->excl_ik[2 * j + 1];
      const real msc = s->excl_scale[4 * j] - 1;
      if (msc == 0)
         continue;
      real xr, yr, zr;
      const real r2 = pair_r(s, im, i, k, xr, yr, zr);
      if (r2 > off2)
         continue;
      real e = 0;
      PairMPoleGrad pg;
      zero(pg);
      pair_mpole<true, false, NON_EWALD>(r2, xr, yr, zr, msc, RP(i), RP(k), f, 0, e, pg);
      etot += e;
   }
   return etot;
}

// order-5 B-spline weights and three derivatives of one fractional offset:
// theta[5][4] (value, d1, d2, d3 per point), the reference's thetai layout
void ref_bsplgen(double w, double* theta)
{
   bsplgen<4>(w, theta, 5);
}

}  // extern "C"
