// C ABI (include/t9gb.h): context lifetime, topology and coordinate upload,
// and the public entry points.  Nothing here allocates inside the hot path:
// every buffer is sized once in t9gb_create from the atom count.
#include <cmath>
#include <cstring>
#include <new>

#include "common.cuh"
#include "reduce.cuh"


namespace t9gb {
int induce_sorted(Context* ctx);
int public_dfield(Context* ctx, float* field, float* fieldp);
int public_ufield(Context* ctx, const float* uind, const float* uinp, float* field, float* fieldp);
int public_precond(Context* ctx, const float* rsd, const float* rsdp, float* zrsd, float* zrsdp);

int stage_dipoles(Context* ctx)
{
   const int n = ctx->n;
   T9_CHECK(scatter_from_sorted3(ctx, ctx->uind, ctx->hout, ctx->hout + 3 * n));
   T9_CUDA(cudaMemcpyAsync(ctx->h_stage, ctx->hout, sizeof(float) * 6 * n, cudaMemcpyDeviceToHost, ctx->stream));
   return T9GB_OK;
}
}  // namespace t9gb

using namespace t9gb;

static int alloc_all(Context* ctx)
{
   const int n = ctx->n, npad = ctx->npad;
   T9_CUDA(cudaMalloc(&ctx->frames, sizeof(int4) * n));
   T9_CUDA(cudaMalloc(&ctx->pole, sizeof(float) * 10 * n));
   T9_CUDA(cudaMalloc(&ctx->xyz, sizeof(float) * 3 * n));
   T9_CUDA(cudaMalloc(&ctx->spos, sizeof(float4) * npad));
   T9_CUDA(cudaMalloc(&ctx->spolar, sizeof(float) * npad));
   T9_CUDA(cudaMalloc(&ctx->spolinv, sizeof(float) * npad));
   T9_CUDA(cudaMalloc(&ctx->sdamp, sizeof(float2) * npad));
   T9_CUDA(cudaMalloc(&ctx->srpole, sizeof(float) * 12 * npad));
   T9_CUDA(cudaMemset(ctx->srpole, 0, sizeof(float) * 12 * npad));
   T9_CUDA(cudaMalloc(&ctx->exfld, sizeof(float) * 4));
   T9_CUDA(cudaMemset(ctx->exfld, 0, sizeof(float) * 4));
   T9_CUDA(cudaMalloc(&ctx->nnbr, sizeof(int) * npad));
   T9_CUDA(cudaMemset(ctx->nnbr, 0, sizeof(int) * npad));
   T9_CUDA(cudaMalloc(&ctx->nnbrc, sizeof(int) * npad));
   T9_CUDA(cudaMemset(ctx->nnbrc, 0, sizeof(int) * npad));
   T9_CUDA(cudaMalloc(&ctx->nnbrp, sizeof(int) * npad));
   T9_CUDA(cudaMemset(ctx->nnbrp, 0, sizeof(int) * npad));
   T9_CUDA(cudaMalloc(&ctx->nbr_over, sizeof(int)));
   T9_CUDA(cudaMemset(ctx->nbr_over, 0, sizeof(int)));
   T9_CUDA(cudaMalloc(&ctx->copy_err, sizeof(int)));
   T9_CUDA(cudaMemset(ctx->copy_err, 0, sizeof(int)));
   T9_CUDA(cudaMallocHost(&ctx->h_over, sizeof(int)));
   *ctx->h_over = 0;
   T9_CUDA(cudaMalloc(&ctx->cell_atoms, sizeof(int) * npad));
   T9_CUDA(cudaMalloc(&ctx->atom_cell, sizeof(int) * npad));
   float** v6[] = {&ctx->rcp6, &ctx->fld6, &ctx->udir, &ctx->efield, &ctx->uind, &ctx->rsd, &ctx->zrsd,
      &ctx->conj, &ctx->vec, &ctx->tmp6};
   for (float** p : v6) {
      T9_CUDA(cudaMalloc(p, sizeof(float) * 8 * npad));
      T9_CUDA(cudaMemset(*p, 0, sizeof(float) * 8 * npad));
   }
   T9_CUDA(cudaMalloc(&ctx->e_atom, sizeof(double) * 3 * npad));
   T9_CUDA(cudaMalloc(&ctx->sframe, sizeof(float) * 9 * npad));
   T9_CUDA(cudaMalloc(&ctx->sref, sizeof(float4) * npad));
   T9_CUDA(cudaMemset(ctx->sref, 0, sizeof(float4) * npad));
   T9_CUDA(cudaMalloc(&ctx->lflag, sizeof(int)));
   T9_CUDA(cudaMemset(ctx->lflag, 0, sizeof(int)));
   T9_CUDA(cudaMallocHost(&ctx->h_lflag, sizeof(int)));
   T9_CUDA(cudaMalloc(&ctx->hout, sizeof(float) * 6 * npad));
   T9_CUDA(cudaMalloc(&ctx->red, sizeof(double) * RED_SLOTS * RED_MAX));
   T9_CUDA(cudaMalloc(&ctx->scal, sizeof(double) * 64));
   T9_CUDA(cudaMemset(ctx->scal, 0, sizeof(double) * 64));
   T9_CUDA(cudaMalloc(&ctx->status, sizeof(int) * 16));
   T9_CUDA(cudaMalloc(&ctx->sum_part, sizeof(double) * SUM_ROWS_MAX * SUM_PARTS));
   T9_CUDA(cudaMemset(ctx->status, 0, sizeof(int) * 16));
   T9_CUDA(cudaMallocHost(&ctx->h_status, sizeof(int) * 16));
   T9_CUDA(cudaMallocHost(&ctx->h_scal, sizeof(double) * 64));
   if (pred_depth(ctx->cfg) > 0) {
      const size_t bytes = sizeof(float) * pred_depth(ctx->cfg) * 8 * (size_t)npad;
      T9_CUDA(cudaMalloc(&ctx->aspc_hist, bytes));
      T9_CUDA(cudaMemset(ctx->aspc_hist, 0, bytes));
   }
   ctx->h_stage_bytes = sizeof(float) * 8 * (size_t)npad;
   T9_CUDA(cudaMallocHost(&ctx->h_stage, ctx->h_stage_bytes));
   T9_CUDA(cudaMallocHost(&ctx->h_in, sizeof(float) * 3 * (size_t)npad));
   T9_CUDA(cudaEventCreateWithFlags(&ctx->ev_in, cudaEventDisableTiming));
   T9_CUDA(cudaEventCreateWithFlags(&ctx->ev_solved, cudaEventDisableTiming));
   for (int k = 0; k < 4; ++k) {
      T9_CUDA(cudaStreamCreateWithFlags(&ctx->side_stream[k], cudaStreamNonBlocking));
      T9_CUDA(cudaEventCreateWithFlags(&ctx->ev_fork[k], cudaEventDisableTiming));
      T9_CUDA(cudaEventCreateWithFlags(&ctx->ev_join[k], cudaEventDisableTiming));
   }
   // the legacy-stream memsets above must finish before work on the caller's
   // (possibly non-blocking) stream
   T9_CUDA(cudaDeviceSynchronize());
   return T9GB_OK;
}

static void free_all(Context* ctx)
{
   void* dev[] = {ctx->frames, ctx->pole, ctx->xyz, ctx->perm, ctx->iperm, ctx->spos, ctx->spolar, ctx->spolinv,
      ctx->sdamp, ctx->srpole, ctx->sp_start, ctx->sp_j, ctx->sp_sc, ctx->nbr, ctx->nnbr, ctx->nbr_over, ctx->nbrc, ctx->nnbrc, ctx->nbrp, ctx->nnbrp,
      ctx->jbl, ctx->jbn, ctx->nbrc_l, ctx->nbrp_l, ctx->copy_err,
      ctx->cell_count, ctx->cell_start, ctx->cell_atoms, ctx->atom_cell, ctx->rcp6, ctx->fld6, ctx->udir,
      ctx->efield, ctx->uind, ctx->rsd, ctx->zrsd, ctx->conj, ctx->vec, ctx->tmp6, ctx->e_atom, ctx->sframe, ctx->hout,
      ctx->red, ctx->scal, ctx->status, ctx->sref, ctx->lflag,
      ctx->aspc_hist, ctx->thl, ctx->exfld, ctx->sum_part, ctx->lx_ab, ctx->lx_part, ctx->lx_coef_buf, ctx->lx_ticket};
   for (void* p : dev)
      if (p)
         cudaFree(p);
   if (ctx->h_status)
      cudaFreeHost(ctx->h_status);
   if (ctx->h_scal)
      cudaFreeHost(ctx->h_scal);
   if (ctx->h_stage)
      cudaFreeHost(ctx->h_stage);
   if (ctx->h_in)
      cudaFreeHost(ctx->h_in);
   if (ctx->ev_in)
      cudaEventDestroy(ctx->ev_in);
   if (ctx->h_over)
      cudaFreeHost(ctx->h_over);
   if (ctx->h_lflag)
      cudaFreeHost(ctx->h_lflag);
   pme_free(ctx);
   learn_free(ctx);
   force_free(ctx);
   vdw_release(ctx);
   valence_release(ctx);
   md_release(ctx);
   drop_graphs(ctx);
   if (ctx->cap_stream)
      cudaStreamDestroy(ctx->cap_stream);
   for (int k = 0; k < 4; ++k) {
      if (ctx->side_stream[k])
         cudaStreamDestroy(ctx->side_stream[k]);
      if (ctx->ev_fork[k])
         cudaEventDestroy(ctx->ev_fork[k]);
      if (ctx->ev_join[k])
         cudaEventDestroy(ctx->ev_join[k]);
   }
   if (ctx->ev_solved)
      cudaEventDestroy(ctx->ev_solved);
   if (ctx->lx_stream)
      cudaStreamDestroy(ctx->lx_stream);
   if (ctx->ev_lx_fork)
      cudaEventDestroy(ctx->ev_lx_fork);
   if (ctx->ev_lx_done)
      cudaEventDestroy(ctx->ev_lx_done);
   for (auto& e : ctx->prof.ev)
      cudaEventDestroy(e);
   if (ctx->own_stream && ctx->stream)
      cudaStreamDestroy(ctx->stream);
}

extern "C" {

const char* t9gb_status_string(int status)
{
   switch (status) {
   case T9GB_OK:
      return "ok";
   case T9GB_NOT_CONVERGED:
      return "induced dipoles are not converged";
   case T9GB_NAN_DETECTED:
      return "non-finite residual in the induced-dipole solve";
   case T9GB_BAD_ARG:
      return "bad argument";
   case T9GB_CUDA_ERR:
      return "CUDA error";
   case T9GB_NO_DEVICE:
      return "no CUDA device";
   case T9GB_NOT_READY:
      return "topology, coordinates or neighbour list missing";
   case T9GB_TOO_LARGE:
      return "input larger than a fixed-capacity entry point or buffer holds";
   default:
      return "unknown status";
   }
}

const char* t9gb_last_error(const t9gb_context* h) { return h ? h->c.last_error.c_str() : "null context"; }

int t9gb_create(const t9gb_config* cfg, t9gb_context** out)
{
   if (!cfg || !out || cfg->n <= 0)
      return T9GB_BAD_ARG;
   *out = nullptr;
   int ndev = 0;
   if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
      return T9GB_NO_DEVICE;
   if (cfg->bsorder != 5 && cfg->use_ewald)
      return T9GB_BAD_ARG;
   const bool pbc = cfg->box[0] > 0 && cfg->box[1] > 0 && cfg->box[2] > 0;
   if (cfg->use_ewald && (!pbc || cfg->nfft[0] < 8 || cfg->nfft[1] < 8 || cfg->nfft[2] < 8 || cfg->aewald <= 0))
      return T9GB_BAD_ARG;
   // ASPC or Gear; the reference's CUDA path has no LSQR predictor
   // (throwExceptionMissingFunction, src/cu/upredict.cu:198-201)
   if (cfg->predictor < 0 || cfg->predictor > 2)
      return T9GB_BAD_ARG;
   if (cfg->politer < 1 || cfg->poleps <= 0)
      return T9GB_BAD_ARG;
   t9gb_context* h = new (std::nothrow) t9gb_context;
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   ctx->cfg = *cfg;
   ctx->n = cfg->n;
   ctx->npad = ((cfg->n + WARP - 1) / WARP) * WARP;
   // lanes per atom of the field kernels: 8 on small boxes, 4 where the box
   // fills the GPU (GB300 induce: 12,288 atoms 0.573 / 0.631 ms at 8 / 4
   // lanes; 98,304 atoms 2.588 / 2.514 ms)
   ctx->pair_lanes = ctx->npad > 32768 ? 4 : 8;
   cudaGetDevice(&ctx->dev);
   int rc = T9GB_OK;
   if (cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess)
      rc = T9GB_CUDA_ERR;
   ctx->own_stream = true;
   if (rc == T9GB_OK)
      rc = alloc_all(ctx);
   if (rc == T9GB_OK)
      rc = pme_setup(ctx);
   if (rc == T9GB_OK)
      rc = pair_staging_setup();
   if (rc == T9GB_OK)
      rc = mlp_tc_setup();
   if (rc != T9GB_OK) {
      free_all(ctx);
      delete h;
      return rc;
   }
   *out = h;
   return T9GB_OK;
}

void t9gb_destroy(t9gb_context* h)
{
   if (!h)
      return;
   cudaStreamSynchronize(h->c.stream);
   if (h->c.lx_stream)
      cudaStreamSynchronize(h->c.lx_stream);
   free_all(&h->c);
   delete h;
}

int t9gb_set_stream(t9gb_context* h, void* stream)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (stream) {
      if (ctx->own_stream && ctx->stream)
         cudaStreamDestroy(ctx->stream);
      ctx->stream = (cudaStream_t)stream;
      ctx->own_stream = false;
   } else if (!ctx->own_stream) {
      T9_CUDA(cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking));
      ctx->own_stream = true;
   }
   return T9GB_OK;
}

int t9gb_set_topology(t9gb_context* h, const int* frames, const double* pole, const double* polarity,
   const double* thole, const double* pdamp, int nexcl, const int* excl_ik, const double* excl_scale)
{
   if (!h || !frames || !pole || !polarity || !thole || !pdamp || nexcl < 0 || (nexcl > 0 && (!excl_ik || !excl_scale)))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   const int n = ctx->n;
   for (int i = 0; i < n; ++i) {
      const int* f = frames + 4 * i;
      if (f[3] < 0 || f[3] > 5)
         return T9GB_BAD_ARG;
      if (f[3] != 0 && (f[0] < 0 || f[0] >= n))
         return T9GB_BAD_ARG;
      if ((f[3] >= 2) && (f[1] < 0 || f[1] >= n))
         return T9GB_BAD_ARG;
      if ((f[3] == 4 || f[3] == 5 || (f[3] == 2 && f[2] != 0)) && (std::abs(f[2]) < 1 || std::abs(f[2]) > n))
         return T9GB_BAD_ARG;
   }
   for (int j = 0; j < nexcl; ++j) {
      int a = excl_ik[2 * j], b = excl_ik[2 * j + 1];
      if (a < 0 || b < 0 || a >= n || b >= n || a == b)
         return T9GB_BAD_ARG;
   }
   ctx->h_polarity.assign(polarity, polarity + n);
   ctx->h_thole.assign(thole, thole + n);
   ctx->h_pdamp.assign(pdamp, pdamp + n);
   ctx->h_excl_ik.assign(excl_ik, excl_ik + 2 * nexcl);
   ctx->h_excl_scale.assign(excl_scale, excl_scale + 4 * nexcl);
   std::vector<float> pf(10 * (size_t)n);
   for (size_t i = 0; i < pf.size(); ++i)
      pf[i] = (float)pole[i];
   T9_CUDA(cudaMemcpy(ctx->frames, frames, sizeof(int4) * n, cudaMemcpyHostToDevice));
   ctx->h_frames.assign(frames, frames + 4 * (size_t)n);
   T9_CUDA(cudaMemcpy(ctx->pole, pf.data(), sizeof(float) * 10 * n, cudaMemcpyHostToDevice));
   T9_CUDA(cudaDeviceSynchronize());  // ordered before work on a non-blocking stream
   ctx->have_topology = true;
   ctx->have_order = false;
   return T9GB_OK;
}

int t9gb_set_thole_pairs(t9gb_context* h, int ntypes, const int* ptype, const double* thlval)
{
   if (!h || ntypes < 0 || ntypes > 256 || (ntypes > 0 && (!ptype || !thlval)))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_topology)
      return T9GB_NOT_READY;
   const int n = ctx->n;
   for (int i = 0; i < n && ntypes > 0; ++i)
      if (ptype[i] < 0 || ptype[i] >= ntypes)
         return T9GB_BAD_ARG;
   std::vector<float> tab((size_t)ntypes * ntypes);
   for (int a = 0; a < ntypes; ++a)
      for (int b = 0; b < ntypes; ++b) {
         const double v = thlval[(size_t)a * ntypes + b];
         // each side of a pair reads its own row: the table must be symmetric
         if (!std::isfinite(v) || v < 0 || v != thlval[(size_t)b * ntypes + a])
            return T9GB_BAD_ARG;
         tab[(size_t)a * ntypes + b] = (float)v;
      }
   if (ctx->thl) {
      T9_CUDA(cudaFree(ctx->thl));
      ctx->thl = nullptr;
   }
   ctx->nthl = 0;
   ctx->h_ptype.clear();
   if (ntypes > 0) {
      T9_CUDA(cudaMalloc(&ctx->thl, sizeof(float) * tab.size()));
      T9_CUDA(cudaMemcpy(ctx->thl, tab.data(), sizeof(float) * tab.size(), cudaMemcpyHostToDevice));
      T9_CUDA(cudaDeviceSynchronize());
      ctx->h_ptype.assign(ptype, ptype + n);
      ctx->nthl = ntypes;
   }
   // the per-slot rows carry the type from the next ordering on
   ctx->have_order = false;
   drop_graphs(ctx);
   return T9GB_OK;
}

int t9gb_set_external_field(t9gb_context* h, const double* field)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   float e[4] = {0.f, 0.f, 0.f, 0.f};
   if (field)
      for (int d = 0; d < 3; ++d) {
         if (!std::isfinite(field[d]))
            return T9GB_BAD_ARG;
         e[d] = (float)field[d];
      }
   // stream-ordered: solves already queued keep the field they were queued
   // with; the pageable source is consumed before the call returns
   for (int d = 0; d < 4; ++d)
      ctx->h_exfld[d] = e[d];
   T9_CUDA(cudaMemcpyAsync(ctx->exfld, ctx->h_exfld, sizeof(float) * 4, cudaMemcpyHostToDevice, ctx->stream));
   ctx->use_exfld = e[0] != 0.f || e[1] != 0.f || e[2] != 0.f;
   return T9GB_OK;
}

int t9gb_set_xyz_host(t9gb_context* h, const double* xyz)
{
   if (!h || !xyz)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   const int n = ctx->n;
   // the previous copy out of the staging buffer must have finished
   if (ctx->ev_in_pending)
      T9_CUDA(cudaEventSynchronize(ctx->ev_in));
   // one pass: convert and check finiteness (exponent field not all ones),
   // four independent integer accumulators so the loop vectorizes
   float* st = ctx->h_in;
   const int m = 3 * n;
   constexpr uint64_t EXP = 0x7ff0000000000000ull;
   uint64_t bad[4] = {0, 0, 0, 0};
   int i = 0;
   for (; i + 4 <= m; i += 4)
      for (int k = 0; k < 4; ++k) {
         const double v = xyz[i + k];
         uint64_t b;
         std::memcpy(&b, &v, sizeof b);
         bad[k] |= (b & EXP) == EXP;
         st[i + k] = (float)v;
      }
   for (; i < m; ++i) {
      const double v = xyz[i];
      uint64_t b;
      std::memcpy(&b, &v, sizeof b);
      bad[0] |= (b & EXP) == EXP;
      st[i] = (float)v;
   }
   if (bad[0] | bad[1] | bad[2] | bad[3])
      return T9GB_BAD_ARG;
   T9_CUDA(cudaMemcpyAsync(ctx->xyz, st, sizeof(float) * 3 * n, cudaMemcpyHostToDevice, ctx->stream));
   T9_CUDA(cudaEventRecord(ctx->ev_in, ctx->stream));
   ctx->ev_in_pending = true;
   ctx->have_xyz = true;
   if (ctx->have_order)
      T9_CHECK(scatter_positions(ctx));
   return T9GB_OK;
}

int t9gb_set_xyz_device(t9gb_context* h, const float* xyz_device)
{
   if (!h || !xyz_device)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   T9_CUDA(cudaMemcpyAsync(ctx->xyz, xyz_device, sizeof(float) * 3 * ctx->n, cudaMemcpyDeviceToDevice, ctx->stream));
   ctx->have_xyz = true;
   if (ctx->have_order)
      T9_CHECK(scatter_positions(ctx));
   return T9GB_OK;
}

int t9gb_nblist_build(t9gb_context* h)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_topology || !ctx->have_xyz)
      return T9GB_NOT_READY;
   {
      // the ordering uses the current device coordinates
      std::vector<float> tmp(3 * (size_t)ctx->n);
      T9_CUDA(cudaMemcpyAsync(tmp.data(), ctx->xyz, sizeof(float) * 3 * ctx->n, cudaMemcpyDeviceToHost, ctx->stream));
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
      ctx->h_xyz.assign(tmp.begin(), tmp.end());
   }
   T9_CHECK(order_build(ctx));
   T9_CHECK(scatter_positions(ctx));
   return T9GB_OK;
}

int t9gb_mpole_init(t9gb_context* h)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   return rotpole_sorted(ctx);
}

int t9gb_dfield(t9gb_context* h, float* field, float* fieldp)
{
   if (!h || !field || !fieldp)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   return public_dfield(ctx, field, fieldp);
}

int t9gb_ufield(t9gb_context* h, const float* uind, const float* uinp, float* field, float* fieldp)
{
   if (!h || !uind || !uinp || !field || !fieldp)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   return public_ufield(ctx, uind, uinp, field, fieldp);
}

int t9gb_sparse_precond_apply(t9gb_context* h, const float* rsd, const float* rsdp, float* zrsd, float* zrsdp)
{
   if (!h || !rsd || !rsdp || !zrsd || !zrsdp)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order || !ctx->cfg.pcgprec)
      return T9GB_NOT_READY;
   return public_precond(ctx, rsd, rsdp, zrsd, zrsdp);
}

int t9gb_induce(t9gb_context* h, float* uind, float* uinp)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   // the caller-order copy rides in the solve's synchronisation
   ctx->out_d = uind;
   ctx->out_p = uinp;
   const int st = induce_sorted(ctx);
   ctx->out_d = ctx->out_p = nullptr;
   return st;
}

int t9gb_induce_host(t9gb_context* h, const double* xyz, double* uind, double* uinp)
{
   if (!h || !xyz)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   T9_CHECK(t9gb_set_xyz_host(h, xyz));
   if (!ctx->have_order)
      T9_CHECK(t9gb_nblist_build(h));
   T9_CHECK(t9gb_mpole_init(h));
   // the dipoles' caller-order copy rides in the solve's synchronisation
   ctx->stage_out = true;
   int st = induce_sorted(ctx);
   ctx->stage_out = false;
   if (st != T9GB_OK && st != T9GB_NOT_CONVERGED && st != T9GB_NAN_DETECTED)
      return st;
   const int m = 3 * ctx->n;
   const float* hs = ctx->h_stage;
   if (uind)
      for (int i = 0; i < m; ++i)
         uind[i] = hs[i];
   if (uinp)
      for (int i = 0; i < m; ++i)
         uinp[i] = hs[m + i];
   return st;
}

int t9gb_induce_stats(const t9gb_context* h, int* iterations, double* eps, int* status)
{
   if (!h)
      return T9GB_BAD_ARG;
   if (iterations)
      *iterations = h->c.last_iter;
   if (eps)
      *eps = h->c.last_eps;
   if (status)
      *status = h->c.last_status;
   return T9GB_OK;
}

int t9gb_get_udir(t9gb_context* h, float* udir, float* udirp)
{
   if (!h || (!udir && !udirp))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   return scatter_from_sorted3(ctx, ctx->udir, udir, udirp);
}

int t9gb_get_uind(t9gb_context* h, float* uind, float* uinp)
{
   if (!h || (!uind && !uinp))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   return scatter_from_sorted3(ctx, ctx->uind, uind, uinp);
}

int t9gb_use_graph(t9gb_context* h, int enable)
{
   if (!h)
      return T9GB_BAD_ARG;
   h->c.use_graph = enable != 0;
   return T9GB_OK;
}

int t9gb_nblist_stats(t9gb_context* h, int* capacity, long long* entries, int* nscaled)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (capacity)
      *capacity = ctx->nbr_cap;
   if (nscaled)
      *nscaled = ctx->nsp / 2;
   if (entries) {
      *entries = 0;
      if (ctx->have_order && !ctx->list_need_build) {
         std::vector<int> cnt(ctx->npad);
         T9_CUDA(cudaMemcpyAsync(cnt.data(), ctx->nnbr, sizeof(int) * ctx->npad, cudaMemcpyDeviceToHost, ctx->stream));
         T9_CUDA(cudaStreamSynchronize(ctx->stream));
         for (int c : cnt)
            *entries += c;
      }
   }
   return T9GB_OK;
}

int t9gb_learn_config(t9gb_context* h, int mode, double lr, double weight_decay)
{
   if (!h || mode < 0 || mode > 3 || !(lr >= 0) || !(weight_decay >= 0))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (mode)
      T9_CHECK(learn_setup(ctx));
   if (mode != ctx->learn_mode || (float)lr != ctx->learn_lr || (float)weight_decay != ctx->learn_wd)
      drop_graphs(ctx);  // the graphs hold the mode, rate and decay
   if ((mode & 2) && !(ctx->learn_mode & 2))
      ctx->learn_since_probe = 1 << 30;  // first solve compares both starts
   ctx->learn_mode = mode;
   ctx->learn_lr = (float)lr;
   ctx->learn_wd = (float)weight_decay;
   return T9GB_OK;
}

int t9gb_pair_lanes(t9gb_context* h, int lanes)
{
   if (!h || (lanes != 4 && lanes != 8 && lanes != 16 && lanes != 32))
      return T9GB_BAD_ARG;
   if (lanes != h->c.pair_lanes)
      drop_graphs(&h->c);
   h->c.pair_lanes = lanes;
   return T9GB_OK;
}

int t9gb_force_lanes(t9gb_context* h, int lanes)
{
   if (!h || (lanes != 4 && lanes != 8 && lanes != 16))
      return T9GB_BAD_ARG;
   h->c.force_lanes = lanes;
   return T9GB_OK;
}

int t9gb_set_pcg_fusion(t9gb_context* h, int mask)
{
   if (!h || mask < 0 || mask > 127)
      return T9GB_BAD_ARG;
   if (mask != h->c.pcg_fuse)
      drop_graphs(&h->c);
   h->c.pcg_fuse = mask;
   return T9GB_OK;
}

int t9gb_pme_fft_cluster(t9gb_context* h, int ctas)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   const int n = ctx->pme.n1;
   if (!(ctas == 0 || ((ctas == 2 || ctas == 4 || (ctas == 8 && n >= 64)) && ctx->pme.own_fft_ok)))
      return T9GB_BAD_ARG;
   if (ctas != ctx->pme.fft_cl)
      drop_graphs(ctx);
   ctx->pme.fft_cl = ctas;
   return T9GB_OK;
}

int t9gb_copy_error(t9gb_context* h, int* flag)
{
   if (!h || !flag)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   int a = 0, b = 0;
   T9_CUDA(cudaMemcpyAsync(&a, ctx->copy_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
   if (ctx->pme.fft_err)
      T9_CUDA(cudaMemcpyAsync(&b, ctx->pme.fft_err, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   *flag = (a & 5) | (b ? 2 : 0);
   return T9GB_OK;
}

int t9gb_learn_extrapolation(t9gb_context* h, int order)
{
   if (!h)
      return T9GB_BAD_ARG;
   return lx_config(&h->c, order);
}

int t9gb_learn_extrapolation_state(t9gb_context* h, int* fits, int* rejected, float* coef16)
{
   if (!h)
      return T9GB_BAD_ARG;
   return lx_state(&h->c, fits, rejected, coef16);
}

int t9gb_learn_tensor_path(t9gb_context* h, int path)
{
   if (!h || (path != 0 && path != 1))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if ((path == 1) != ctx->mlp_tc)
      drop_graphs(ctx);
   ctx->mlp_tc = path == 1;
   return T9GB_OK;
}

int t9gb_pair_staging(t9gb_context* h, int enable)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if ((enable != 0) != ctx->pair_staged) {
      drop_graphs(ctx);
      // the staged kernels read the local indices and j-block lists of the
      // latest staging filter pass: refilter before the next field, and
      // until then no block is staged
      if (ctx->jbn)
         T9_CUDA(cudaMemsetAsync(ctx->jbn, 0x7f, sizeof(int) * (size_t)(ctx->npad / 32), ctx->stream));
      ctx->list_stale = true;
   }
   ctx->pair_staged = enable != 0;
   return T9GB_OK;
}

int t9gb_pme_own_fft(t9gb_context* h, int enable)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (enable && !ctx->pme.own_fft_ok)
      return T9GB_BAD_ARG;
   if ((enable != 0) != ctx->pme.own_fft)
      drop_graphs(ctx);
   ctx->pme.own_fft = enable != 0;
   return T9GB_OK;
}

int t9gb_learn_policy(t9gb_context* h, int probe_every)
{
   if (!h || probe_every < 1)
      return T9GB_BAD_ARG;
   h->c.learn_probe = probe_every;
   h->c.learn_since_probe = 1 << 30;
   return T9GB_OK;
}

int t9gb_learn_reset(t9gb_context* h, unsigned seed)
{
   if (!h)
      return T9GB_BAD_ARG;
   return learn_reset(&h->c, seed);
}

int t9gb_learn_stats(t9gb_context* h, int* choice, double* eps0_plain, double* eps0_learned, double* loss,
   int* compared)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   const double* sc = ctx->h_scal;
   const double n = std::max(1, ctx->n), debye = ctx->cfg.debye;
   if (choice)
      *choice = (ctx->learn_mode & 2) ? ctx->h_status[ST_LCHOICE] : 0;
   if (eps0_plain)
      *eps0_plain = debye * std::sqrt(std::max(sc[S_L_PLAIN_D], sc[S_L_PLAIN_P]) / n);
   if (eps0_learned)
      *eps0_learned = debye * std::sqrt(std::max(sc[S_L_LEARN_D], sc[S_L_LEARN_P]) / n);
   if (loss)
      *loss = sc[S_L_LOSS];
   if (compared)
      *compared = ctx->learn_variant == 2 ? 1 : 0;
   return T9GB_OK;
}

int t9gb_learn_get_weights(t9gb_context* h, float* w, int nparam)
{
   if (!h || !w || nparam != T9GB_LEARN_NPARAM)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   T9_CHECK(learn_setup(ctx));
   return mlp_get_weights(ctx, w);
}

int t9gb_learn_set_weights(t9gb_context* h, const float* w, int nparam)
{
   if (!h || !w || nparam != T9GB_LEARN_NPARAM)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   T9_CHECK(learn_setup(ctx));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return mlp_set_weights(ctx, w);
}

int t9gb_learn_eval(t9gb_context* h, int rows, const float* x, const float* t, float* y, float* grad, double* loss)
{
   if (!h || rows <= 0 || !x || !t)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   T9_CHECK(learn_setup(ctx));
   MlpState& S = ctx->mlp;
   if (rows > S.max_rows) {
      ctx->last_error = "more rows than the network's buffers hold (2 x the atom count rounded up to 32)";
      return T9GB_TOO_LARGE;
   }
   std::vector<__nv_bfloat16> xb((size_t)rows * MLP_IN);
   for (size_t i = 0; i < xb.size(); ++i)
      xb[i] = __float2bfloat16(x[i]);
   cudaStream_t st = ctx->stream;
   T9_CUDA(cudaMemcpyAsync(S.x, xb.data(), sizeof(__nv_bfloat16) * xb.size(), cudaMemcpyHostToDevice, st));
   T9_CUDA(cudaMemcpyAsync(S.t, t, sizeof(float) * rows * MLP_OUT, cudaMemcpyHostToDevice, st));
   T9_CHECK(mlp_forward(ctx, rows));
   T9_CHECK(mlp_backward(ctx, rows, nullptr, 0));
   std::vector<float> yy((size_t)rows * MLP_OUT_PAD);
   double l = 0;
   T9_CUDA(cudaMemcpyAsync(yy.data(), S.y, sizeof(float) * yy.size(), cudaMemcpyDeviceToHost, st));
   if (grad)
      T9_CUDA(cudaMemcpyAsync(grad, S.g, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, st));
   T9_CUDA(cudaMemcpyAsync(&l, S.loss, sizeof(double), cudaMemcpyDeviceToHost, st));
   T9_CUDA(cudaStreamSynchronize(st));
   if (y)
      for (int r = 0; r < rows; ++r)
         for (int c = 0; c < MLP_OUT; ++c)
            y[r * MLP_OUT + c] = yy[(size_t)r * MLP_OUT_PAD + c];
   if (loss)
      *loss = l / ((double)rows * MLP_OUT);
   return T9GB_OK;
}

int t9gb_learn_adamw(t9gb_context* h)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   T9_CHECK(learn_setup(ctx));
   T9_CHECK(mlp_adamw(ctx, ctx->learn_lr, ctx->learn_wd));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return T9GB_OK;
}

int t9gb_learn_features(t9gb_context* h, float* features_device)
{
   if (!h || !features_device)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->xf || !ctx->have_order)
      return T9GB_NOT_READY;
   return learn_features_out(ctx, features_device);
}

int t9gb_profile_enable(t9gb_context* h, int enable)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   Profiler& p = ctx->prof;
   if (enable && p.ev.empty()) {
      const int npair = 8192;
      p.ev.resize(2 * npair);
      p.cat.resize(npair);
      for (auto& e : p.ev)
         T9_CUDA(cudaEventCreate(&e));
   }
   p.on = enable != 0;
   p.used = 0;
   return T9GB_OK;
}

int t9gb_profile_read(t9gb_context* h, int category, double* total_ms, long long* launches, int reset)
{
   if (!h || category < 0 || category >= P_NCAT)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   prof_collect(ctx);
   if (total_ms)
      *total_ms = ctx->prof.ms[category];
   if (launches)
      *launches = ctx->prof.cnt[category];
   if (reset) {
      ctx->prof.ms[category] = 0;
      ctx->prof.cnt[category] = 0;
   }
   return T9GB_OK;
}

const char* t9gb_profile_name(int category)
{
   static const char* names[P_NCAT] = {"dfield_real", "ufield_real", "precond_sparse", "spread_mpole",
      "spread_uind", "fft_conv", "gather_mpole", "gather_uind", "pcg_vector", "nblist"};
   if (category < 0 || category >= P_NCAT)
      return "";
   return names[category];
}

}  // extern "C"
