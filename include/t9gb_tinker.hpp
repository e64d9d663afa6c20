/*
 * t9gb_tinker.hpp -- the reference's C++ entry points for the AMOEBA
 * polarization path, with the reference's names and signatures, forwarding
 * to the C ABI in t9gb.h.
 *
 * A Tinker9 build (TinkerTools/tinker-gpu) links libt9gb_tinker.so in place
 * of the CUDA implementations of these routines; its DYNAMIC / ANALYZE
 * drivers call them unchanged.  Mixed precision with deterministic forces:
 * real = float, grad_prec = fixed (unsigned 64-bit at 2^32 per kcal/mol/A).
 *
 * State.  The reference keeps its inputs and outputs in module globals
 * (TINKER_EXTERN in include/ff/atom.h, include/ff/modamoeba.h,
 * include/tool/rcman.h).  This header declares the ones these routines read
 * and write, with the reference's names and types.  Inside a Tinker9 build
 * they are the reference's own definitions (define
 * T9GB_TINKER_EXTERNAL_GLOBALS so the library does not define them a second
 * time); standalone, libt9gb_tinker.so defines them.  The library context is
 * bound once with t9gbBind (the RcOp::ALLOC/INIT step of epolarData /
 * empoleData, src/amoeba/epolar.cpp:486-508).
 *
 * Errors.  Every failing status becomes tinker::FatalError, the exception
 * TINKER_THROW raises (include/tool/error.h:15-44): non-convergence of the
 * dipoles throws like src/cu/amoeba/pcg.cu:180-184.
 */
#ifndef T9GB_TINKER_HPP
#define T9GB_TINKER_HPP

#include <exception>
#include <string>

#include "t9gb.h"

namespace tinker {
#ifndef T9GB_TINKER_HAVE_TYPES
/* include/ff/precision.h:68-106, TINKER_MIXED_PRECISION with
 * TINKER_DETERMINISTIC_FORCE */
typedef float real;
typedef double mixed;
typedef unsigned long long fixed;
typedef fixed grad_prec;
typedef mixed energy_prec;
typedef mixed virial_prec;

/* include/tool/error.h:15-36 */
class FatalError : public std::exception
{
   std::string m_msg;

public:
   explicit FatalError(const char* msg) : m_msg(msg) {}
   explicit FatalError(const std::string& msg) : m_msg(msg) {}
   const char* what() const noexcept override { return m_msg.c_str(); }
};

/* include/tool/rcman.h:105-155 */
struct calc
{
   static constexpr int xyz = 0x001;
   static constexpr int energy = 0x010;
   static constexpr int grad = 0x020;
   static constexpr int virial = 0x040;
   static constexpr int analyz = 0x080;
   static constexpr int md = 0x100;
   static constexpr int vmask = energy + grad + virial + analyz;
   static constexpr int v0 = energy;
   static constexpr int v1 = energy + grad + virial;
   static constexpr int v3 = energy + analyz;
   static constexpr int v4 = energy + grad;
   static constexpr int v5 = grad;
   static constexpr int v6 = grad + virial;
};
#endif

/* ---- module globals read and written by these routines ---- */
extern int n;                          /* include/ff/atom.h:40 */
extern real *x, *y, *z;                /* include/ff/atom.h:43-45, device */
extern int rc_flag;                    /* include/tool/rcman.h:183 */
extern real (*uind)[3], (*uinp)[3];    /* include/ff/modamoeba.h:51-52, device */
extern real (*udir)[3], (*udirp)[3];   /* include/ff/modamoeba.h:49-50, device */
extern grad_prec *demx, *demy, *demz;  /* include/ff/modamoeba.h:19-21, device */
extern grad_prec *depx, *depy, *depz;  /* include/ff/modamoeba.h:57-59, device */
extern energy_prec energy_em, energy_ep;          /* modamoeba.h:22,60 */
extern virial_prec virial_em[9], virial_ep[9];    /* modamoeba.h:23,61 */

/* Bind the library context whose topology, settings and stream these
 * routines use (the caller created it with t9gb_create + t9gb_set_topology,
 * the reference's epolarData / empoleData / pmeData INIT).  Allocates the
 * routines' float gradient scratch [n][3] on the context's device. */
void t9gbBind(t9gb_context* ctx);
/* Releases the scratch (RcOp::DEALLOC). */
void t9gbUnbind();
t9gb_context* t9gbContext();

/* include/ff/amoeba/induce.h:8-34 */
void dfield(real (*field)[3], real (*fieldp)[3]);
void ufield(const real (*uind)[3], const real (*uinp)[3], real (*field)[3], real (*fieldp)[3]);
void diagPrecond(const real (*rsd)[3], const real (*rsdp)[3], real (*zrsd)[3], real (*zrsdp)[3]);
void sparsePrecondApply(const real (*rsd)[3], const real (*rsdp)[3], real (*zrsd)[3], real (*zrsdp)[3]);
void induce(real (*uind)[3], real (*uinp)[3]);

/* include/ff/amoeba/empole.h:10-13: coordinates from x, y, z, then the
 * local -> global rotation of the multipoles (chkpole + rotpole). */
void mpoleInit(int vers);

/* include/ff/amoeba/empole.h:11, epolar.h:10, emplar.h:14.  Energies go to
 * energy_em / energy_ep, virials to virial_em / virial_ep, gradients (fixed
 * point) are added to demx.. / depx..; with rc_flag & calc::analyz the
 * gradient arrays are zeroed first, as the reference does for a standalone
 * evaluation.  emplar puts the whole multipole + polarization gradient and
 * virial into dem* / virial_em (the reference's emplar_cu writes its fused
 * real-space pass to dem* / vir_em and the reciprocal polarization part to
 * dep*; the drivers only use their sum), the multipole energy into
 * energy_em and the polarization energy into energy_ep.  The calc::analyz
 * interaction counts (nem, nep) are not produced. */
void empole(int vers);
void epolar(int vers);
void emplar(int vers);
}

#endif
