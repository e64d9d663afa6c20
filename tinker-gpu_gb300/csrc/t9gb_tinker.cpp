// The reference's C++ entry points for the AMOEBA polarization path
// (namespace tinker, the signatures of include/ff/amoeba/{induce,empole,
// epolar,emplar}.h), forwarding to the C ABI.  Host C++ only: the device
// work is all behind t9gb.h.
#include "t9gb_tinker.hpp"

#include <cuda_runtime_api.h>

#include <string>

namespace tinker {
#ifndef T9GB_TINKER_EXTERNAL_GLOBALS
int n = 0;
real *x = nullptr, *y = nullptr, *z = nullptr;
int rc_flag = 0;
real (*uind)[3] = nullptr;
real (*uinp)[3] = nullptr;
real (*udir)[3] = nullptr;
real (*udirp)[3] = nullptr;
grad_prec *demx = nullptr, *demy = nullptr, *demz = nullptr;
grad_prec *depx = nullptr, *depy = nullptr, *depz = nullptr;
energy_prec energy_em = 0, energy_ep = 0;
virial_prec virial_em[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
virial_prec virial_ep[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
#endif

namespace {
t9gb_context* g_ctx = nullptr;
float* g_grad = nullptr;  // [n][3] float gradient of the last term
bool g_ordered = false;   // the spatial order has been built

[[noreturn]] void fail(const char* where, int rc)
{
   std::string m = std::string(where) + ": " + t9gb_status_string(rc);
   if (g_ctx) {
      const char* detail = t9gb_last_error(g_ctx);
      if (detail && *detail)
         m += std::string(" (") + detail + ")";
   }
   throw FatalError(m);
}

void check(const char* where, int rc)
{
   if (rc != T9GB_OK)
      fail(where, rc);
}

t9gb_context* ctx_or_throw(const char* where)
{
   if (!g_ctx)
      throw FatalError(std::string(where) + ": no library context bound (call tinker::t9gbBind)");
   return g_ctx;
}

void zero_grad(grad_prec* gx, grad_prec* gy, grad_prec* gz)
{
   // no source gradient: the words are cleared, in the context's stream order
   check("zero gradient", t9gb_gradient_fixed(g_ctx, nullptr, 0, gx, gy, gz));
}

using TermFn = int (*)(t9gb_context*, int, double*, float*, double*);

// one energy term: the C-ABI call, then the reference's outputs
void term(const char* where, TermFn fn, int vers, energy_prec* e_out, virial_prec* v_out, grad_prec* gx,
   grad_prec* gy, grad_prec* gz)
{
   t9gb_context* ctx = ctx_or_throw(where);
   const int v = vers & (calc::energy | calc::grad | calc::virial);
   const bool do_g = (v & calc::grad) != 0;
   const bool do_v = (v & calc::virial) != 0;
   *e_out = 0;
   for (int k = 0; k < 9; ++k)
      v_out[k] = 0;
   if (do_g && (rc_flag & calc::analyz))
      zero_grad(gx, gy, gz);
   mpoleInit(vers);
   if (!v)
      return;
   double e = 0, w[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
   const int rc = fn(ctx, v, &e, do_g ? g_grad : nullptr, do_v ? w : nullptr);
   if (rc != T9GB_OK)
      fail(where, rc);
   if (do_g)
      check(where, t9gb_gradient_fixed(ctx, g_grad, 1, gx, gy, gz));
   if (v & calc::energy)
      *e_out = e;
   if (do_v)
      for (int k = 0; k < 9; ++k)
         v_out[k] = w[k];
}
}  // namespace

void t9gbBind(t9gb_context* ctx)
{
   t9gbUnbind();
   if (!ctx)
      throw FatalError("t9gbBind: null context");
   if (n <= 0)
      throw FatalError("t9gbBind: tinker::n is not set");
   if (cudaMalloc((void**)&g_grad, sizeof(float) * 3 * (size_t)n) != cudaSuccess) {
      g_grad = nullptr;
      throw FatalError("t9gbBind: cudaMalloc of the gradient scratch failed");
   }
   g_ctx = ctx;
   g_ordered = false;
}

void t9gbUnbind()
{
   if (g_grad)
      cudaFree(g_grad);
   g_grad = nullptr;
   g_ctx = nullptr;
   g_ordered = false;
}

t9gb_context* t9gbContext() { return g_ctx; }

void mpoleInit(int)
{
   t9gb_context* ctx = ctx_or_throw("mpoleInit");
   check("mpoleInit", t9gb_set_xyz_soa_device(ctx, x, y, z));
   if (!g_ordered) {
      check("mpoleInit", t9gb_nblist_build(ctx));
      g_ordered = true;
   }
   check("mpoleInit", t9gb_mpole_init(ctx));
}

void dfield(real (*field)[3], real (*fieldp)[3])
{
   check("dfield", t9gb_dfield(ctx_or_throw("dfield"), &field[0][0], &fieldp[0][0]));
}

void ufield(const real (*uind_)[3], const real (*uinp_)[3], real (*field)[3], real (*fieldp)[3])
{
   check("ufield", t9gb_ufield(ctx_or_throw("ufield"), &uind_[0][0], &uinp_[0][0], &field[0][0], &fieldp[0][0]));
}

void diagPrecond(const real (*rsd)[3], const real (*rsdp)[3], real (*zrsd)[3], real (*zrsdp)[3])
{
   check("diagPrecond", t9gb_diag_precond_apply(ctx_or_throw("diagPrecond"), &rsd[0][0],
                           rsdp ? &rsdp[0][0] : nullptr, &zrsd[0][0], zrsdp ? &zrsdp[0][0] : nullptr));
}

void sparsePrecondApply(const real (*rsd)[3], const real (*rsdp)[3], real (*zrsd)[3], real (*zrsdp)[3])
{
   check("sparsePrecondApply", t9gb_sparse_precond_apply(ctx_or_throw("sparsePrecondApply"), &rsd[0][0],
                                  &rsdp[0][0], &zrsd[0][0], &zrsdp[0][0]));
}

void induce(real (*uind_)[3], real (*uinp_)[3])
{
   t9gb_context* ctx = ctx_or_throw("induce");
   const int rc = t9gb_induce(ctx, &uind_[0][0], &uinp_[0][0]);
   if (rc == T9GB_NOT_CONVERGED) {
      int it = 0;
      double eps = 0;
      t9gb_induce_stats(ctx, &it, &eps, nullptr);
      throw FatalError("PCG Induced Dipoles are not converged after " + std::to_string(it) +
         " iterations, RMS residual " + std::to_string(eps) + " Debye");
   }
   check("induce", rc);
   if (udir && udirp)
      check("induce", t9gb_get_udir(ctx, &udir[0][0], &udirp[0][0]));
}

void empole(int vers)
{
   term("empole", t9gb_empole, vers, &energy_em, virial_em, demx, demy, demz);
}

void epolar(int vers)
{
   term("epolar", t9gb_epolar, vers, &energy_ep, virial_ep, depx, depy, depz);
   if (uind && uinp)
      check("epolar", t9gb_get_uind(g_ctx, &uind[0][0], &uinp[0][0]));
}

void emplar(int vers)
{
   term("emplar", t9gb_emplar, vers, &energy_em, virial_em, demx, demy, demz);
   energy_ep = 0;
   if (vers & calc::energy) {
      double parts[4];
      check("emplar", t9gb_energy_components(g_ctx, parts));
      energy_em = parts[0] + parts[1] + parts[2];
      energy_ep = parts[3];
   }
   if (uind && uinp)
      check("emplar", t9gb_get_uind(g_ctx, &uind[0][0], &uinp[0][0]));
}
}  // namespace tinker
