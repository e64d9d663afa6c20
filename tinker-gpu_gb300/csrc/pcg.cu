// Preconditioned conjugate gradient for the AMOEBA mutual dipoles, the
// public field entry points, and the ASPC predictor.
//
// Control flow follows induceMutualPcg1_cu (src/cu/amoeba/pcg.cu:14-185) and
// the CG steps documented in include/ff/cuinduce.h:8-35:
//   r0 = E - (1/alpha + T) u0,  p = z = M r0,  s = r.z
//   loop: Ap = p/alpha - ufield(p); a = s / p.Ap; u += a p; r -= a Ap;
//         z = M r; s1 = r.z; p = z + (s1/s) p; s = s1;
//         eps = debye sqrt(max(r.r)/n); stop when eps < poleps (at least 3
//         iterations, at most politer); then u += pcgpeek alpha r.
// The reference runs ~20 launches per iteration including eight cuBLAS Sdot
// calls and a host synchronisation (pcg.cu:144-145).  Here an iteration is
// the ufield chain, the preconditioner and four element-parallel vector
// kernels.  Every dot product is an FP64 block partial that each consumer
// block re-reduces in a fixed order (bit-reproducible); the convergence test
// runs on the device.
#include <cmath>

#include "common.cuh"

namespace t9gb {

// device PCG state (ctx->scal as doubles, ctx->status as ints)
enum { S_SUM_D = 0, S_SUM_P = 1, S_EPS = 2, S_COEF = 8, S_NSCAL = 24 };
enum { ST_ITER = 0, ST_DONE = 1, ST_STATUS = 2, ST_NSTAT = 4 };
// reduction slots
enum { R_PAP_D = 0, R_PAP_P = 1, R_RZ_D = 2, R_RZ_P = 3, R_RR_D = 4, R_RR_P = 5 };

constexpr int VB = 256;  // vector-kernel block size

__device__ double block_sum(double v, double* sh)
{
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
      v += __shfl_down_sync(0xffffffffu, v, o);
   const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
   if (l == 0)
      sh[w] = v;
   __syncthreads();
   double r = 0;
   if (threadIdx.x < 32) {
      r = threadIdx.x < (blockDim.x >> 5) ? sh[threadIdx.x] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         r += __shfl_down_sync(0xffffffffu, r, o);
   }
   __syncthreads();
   return r;  // valid in thread 0
}

// deterministic sum of nb partials, broadcast to the block
__device__ double finalize(const double* part, int nb, double* sh)
{
   double v = 0;
   for (int i = threadIdx.x; i < nb; i += blockDim.x)
      v += part[i];
   v = block_sum(v, sh);
   if (threadIdx.x == 0)
      sh[32] = v;
   __syncthreads();
   double r = sh[32];
   __syncthreads();
   return r;
}

__device__ __forceinline__ void store_partial(double* red, int slot, double v, double* sh)
{
   v = block_sum(v, sh);
   if (threadIdx.x == 0)
      red[slot * RED_MAX + blockIdx.x] = v;
}

struct VecArgs {
   int ne;  // 6 * npad elements
   int nb;  // blocks of every vector kernel (fixed: partial counts match)
   const float* polar;
   const float* polinv;
   int sparse;
};

// ---- start of induce ----

// E = field, udir = alpha E, initial guess (guess 0 zero, 1 direct, 2 ASPC)
__global__ void k_init_guess(VecArgs A, const float* __restrict__ fld, float* __restrict__ efield,
   float* __restrict__ udir, float* __restrict__ uind, int guess, const float* __restrict__ hist,
   const double* __restrict__ coef)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const float pol = A.polar[e / 6];
      const float f = fld[e];
      efield[e] = f;
      const float ud = pol * f;
      udir[e] = ud;
      float u = 0.f;
      if (guess == 1) {
         u = ud;
      } else if (guess == 2) {
         double v = 0;
         for (int k = 0; k < 16; ++k)
            v += coef[k] * (double)hist[(size_t)k * A.ne + e];
         u = (float)v;
      }
      uind[e] = u;
   }
}

// r0 from the guess (fld holds ufield(u0) when guess != 0)
__global__ void k_init_rsd(VecArgs A, const float* __restrict__ fld, const float* __restrict__ efield,
   const float* __restrict__ udir, const float* __restrict__ uind, float* __restrict__ rsd, int guess)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6;
      float r;
      if (guess == 2)
         r = (udir[e] - uind[e]) * A.polinv[s] + fld[e];
      else if (guess == 1)
         r = fld[e];
      else
         r = efield[e];
      if (A.polar[s] == 0.f)
         r = 0.f;
      rsd[e] = r;
   }
}

// z = M r (diagonal here, or read from the sparse kernel); p = z on init;
// partials r.z and r.r
__global__ void k_precond_dot(VecArgs A, const float* __restrict__ rsd, float* __restrict__ zrsd,
   float* __restrict__ conj, double* __restrict__ red, int init)
{
   __shared__ double sh[40];
   double rz_d = 0, rz_p = 0, rr_d = 0, rr_p = 0;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const float r = rsd[e];
      float z;
      if (A.sparse) {
         z = zrsd[e];
      } else {
         z = A.polar[e / 6] * r;
         zrsd[e] = z;
      }
      if (init)
         conj[e] = z;
      if (e % 6 < 3) {
         rz_d += (double)r * z;
         rr_d += (double)r * r;
      } else {
         rz_p += (double)r * z;
         rr_p += (double)r * r;
      }
   }
   store_partial(red, R_RZ_D, rz_d, sh);
   store_partial(red, R_RZ_P, rz_p, sh);
   store_partial(red, R_RR_D, rr_d, sh);
   store_partial(red, R_RR_P, rr_p, sh);
}

// ---- loop body ----

// Ap = p/alpha - ufield(p); partials p.Ap; counts the iteration
__global__ void k_pcg_p1(VecArgs A, const float* __restrict__ fld, const float* __restrict__ conj,
   float* __restrict__ vec, double* __restrict__ red, int* __restrict__ state)
{
   __shared__ double sh[40];
   if (blockIdx.x == 0 && threadIdx.x == 0)
      state[ST_ITER] += 1;
   double dd = 0, dp = 0;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const float p = conj[e];
      const float v = A.polinv[e / 6] * p - fld[e];
      vec[e] = v;
      if (e % 6 < 3)
         dd += (double)p * v;
      else
         dp += (double)p * v;
   }
   store_partial(red, R_PAP_D, dd, sh);
   store_partial(red, R_PAP_P, dp, sh);
}

// a = s / p.Ap; u += a p; r -= a Ap; records s for the b step
__global__ void k_pcg_p2(VecArgs A, const double* __restrict__ red, double* __restrict__ scal,
   float* __restrict__ uind, const float* __restrict__ conj, float* __restrict__ rsd, const float* __restrict__ vec)
{
   __shared__ double sh[40];
   const double pap_d = finalize(red + R_PAP_D * RED_MAX, A.nb, sh);
   const double pap_p = finalize(red + R_PAP_P * RED_MAX, A.nb, sh);
   const double sum_d = finalize(red + R_RZ_D * RED_MAX, A.nb, sh);
   const double sum_p = finalize(red + R_RZ_P * RED_MAX, A.nb, sh);
   if (blockIdx.x == 0 && threadIdx.x == 0) {
      scal[S_SUM_D] = sum_d;
      scal[S_SUM_P] = sum_p;
   }
   const float a = pap_d == 0 ? 0.f : (float)(sum_d / pap_d);
   const float ap = pap_p == 0 ? 0.f : (float)(sum_p / pap_p);
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const float g = e % 6 < 3 ? a : ap;
      uind[e] += g * conj[e];
      float r = rsd[e] - g * vec[e];
      if (A.polar[e / 6] == 0.f)
         r = 0.f;
      rsd[e] = r;
   }
}

// b = s1/s; p = z + b p; convergence test; peek on the last iteration
__global__ void k_pcg_p4(VecArgs A, const double* __restrict__ red, double* __restrict__ scal,
   int* __restrict__ state, float* __restrict__ conj, const float* __restrict__ zrsd, float* __restrict__ uind,
   const float* __restrict__ rsd, int n, double debye, double poleps, int politer, int miniter, float pcgpeek)
{
   __shared__ double sh[40];
   const double s1_d = finalize(red + R_RZ_D * RED_MAX, A.nb, sh);
   const double s1_p = finalize(red + R_RZ_P * RED_MAX, A.nb, sh);
   const double rr_d = finalize(red + R_RR_D * RED_MAX, A.nb, sh);
   const double rr_p = finalize(red + R_RR_P * RED_MAX, A.nb, sh);
   const double s_d = scal[S_SUM_D], s_p = scal[S_SUM_P];
   const float b = s_d == 0 ? 0.f : (float)(s1_d / s_d);
   const float bp = s_p == 0 ? 0.f : (float)(s1_p / s_p);
   const double eps = debye * sqrt(fmax(rr_d, rr_p) / n);
   const int iter = state[ST_ITER];
   bool done = eps < poleps;
   if (iter < miniter)
      done = false;
   if (iter >= politer)
      done = true;
   if (!(eps == eps))  // NaN: stop and report
      done = true;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const float g = e % 6 < 3 ? b : bp;
      conj[e] = zrsd[e] + g * conj[e];
      if (done)
         uind[e] += pcgpeek * A.polar[e / 6] * rsd[e];
   }
   if (blockIdx.x == 0 && threadIdx.x == 0) {
      scal[S_EPS] = eps;
      state[ST_DONE] = done ? 1 : 0;
      int st = T9GB_OK;
      if (!(eps == eps))
         st = T9GB_NAN_DETECTED;
      else if (done && !(eps < poleps))
         st = T9GB_NOT_CONVERGED;
      state[ST_STATUS] = st;
   }
}

__global__ void k_reset_state(int* state, double* scal)
{
   state[ST_ITER] = 0;
   state[ST_DONE] = 0;
   state[ST_STATUS] = 0;
   scal[S_EPS] = 0;
}

__global__ void k_copy(int ne, const float* __restrict__ src, float* __restrict__ dst)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < ne; i += gridDim.x * blockDim.x)
      dst[i] = src[i];
}

// ---------------------------------------------------------------------------

static VecArgs vec_args(const Context* ctx)
{
   VecArgs A;
   A.ne = 6 * ctx->npad;
   A.nb = std::min(RED_MAX, grid_for(A.ne, VB));
   A.polar = ctx->spolar;
   A.polinv = ctx->spolinv;
   A.sparse = ctx->cfg.pcgprec ? 1 : 0;
   return A;
}

// neighbour list for the current coordinates; overflow is checked after the
// caller's final synchronisation (check_list_overflow)
static int ensure_list(Context* ctx)
{
   if (!ctx->list_stale)
      return T9GB_OK;
   T9_CHECK(list_update(ctx));
   T9_CUDA(cudaMemcpyAsync(ctx->h_over, ctx->nbr_over, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
   return T9GB_OK;
}

// after a synchronisation: grow the list if any atom had more neighbours
// than the row capacity; returns 1 when the caller must redo its work
static int check_list_overflow(Context* ctx, int* redo)
{
   *redo = 0;
   if (*ctx->h_over <= ctx->nbr_cap)
      return T9GB_OK;
   int cap = ((int)(*ctx->h_over * 1.25) + 31) / 32 * 32;
   cudaFree(ctx->nbr);
   ctx->nbr = nullptr;
   T9_CUDA(cudaMalloc(&ctx->nbr, sizeof(int) * (size_t)ctx->npad * cap));
   ctx->nbr_cap = cap;
   *ctx->h_over = 0;
   T9_CUDA(cudaMemset(ctx->nbr_over, 0, sizeof(int)));
   ctx->list_stale = true;
   *redo = 1;
   return T9GB_OK;
}

static int ufield6(Context* ctx, const float* u6, float* out6)
{
   T9_CHECK(launch_ufield_recip(ctx, u6, ctx->rcp6));
   T9_CHECK(launch_ufield_real(ctx, u6, ctx->cfg.use_ewald ? ctx->rcp6 : nullptr, out6));
   return T9GB_OK;
}

static int dfield6(Context* ctx, float* out6)
{
   T9_CHECK(launch_dfield_recip(ctx, ctx->rcp6));
   T9_CHECK(launch_dfield_real(ctx, ctx->cfg.use_ewald ? ctx->rcp6 : nullptr, out6));
   return T9GB_OK;
}

// ASPC extrapolation weights (Kolafa, J. Comput. Chem. 25, 335 (2004)); the
// reference tabulates them in src/cu/upredict.cu:40-55.
static const double ASPC[16] = {62. / 17., -310. / 51., 2170. / 323., -2329. / 400., 1701. / 409., -806. / 323.,
   1024. / 809., -479. / 883., 257. / 1316., -434. / 7429., 191. / 13375., -62. / 22287., 3. / 7217.,
   -3. / 67015., 2. / 646323., -1. / 9694845.};

static int pcg_body(Context* ctx, const VecArgs& A)
{
   const t9gb_config& c = ctx->cfg;
   T9_CHECK(ufield6(ctx, ctx->conj, ctx->fld6));
   prof_begin(ctx, P_VECTOR);
   k_pcg_p1<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->fld6, ctx->conj, ctx->vec, ctx->red, ctx->status);
   k_pcg_p2<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->red, ctx->scal, ctx->uind, ctx->conj, ctx->rsd, ctx->vec);
   prof_end(ctx);
   if (A.sparse)
      T9_CHECK(launch_precond_sparse(ctx, ctx->rsd, ctx->zrsd));
   const int miniter = std::min(3, ctx->n);
   prof_begin(ctx, P_VECTOR);
   k_precond_dot<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->rsd, ctx->zrsd, ctx->conj, ctx->red, 0);
   k_pcg_p4<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->red, ctx->scal, ctx->status, ctx->conj, ctx->zrsd, ctx->uind,
      ctx->rsd, ctx->n, c.debye, c.poleps, c.politer, miniter, (float)c.pcgpeek);
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// dfield, guess, r0 and M r0: everything before the loop
static int pcg_start(Context* ctx, const VecArgs& A)
{
   const t9gb_config& c = ctx->cfg;
   int guess = c.pcgguess ? 1 : 0;
   if (c.predictor == 1 && ctx->nualt >= 16) {
      guess = 2;
      double coef[16];
      for (int s = 0; s < 16; ++s)
         coef[s] = ASPC[((ctx->nualt - 1 - s) % 16 + 16) % 16];
      for (int s = 0; s < 16; ++s)
         ctx->h_scal[S_COEF + s] = coef[s];
      T9_CUDA(cudaMemcpyAsync(ctx->scal + S_COEF, ctx->h_scal + S_COEF, sizeof(double) * 16, cudaMemcpyHostToDevice,
         ctx->stream));
   }
   k_reset_state<<<1, 1, 0, ctx->stream>>>(ctx->status, ctx->scal);
   T9_CHECK(ensure_list(ctx));
   T9_CHECK(dfield6(ctx, ctx->fld6));
   k_init_guess<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->fld6, ctx->efield, ctx->udir, ctx->uind, guess,
      ctx->aspc_hist, ctx->scal + S_COEF);
   if (guess != 0)
      T9_CHECK(ufield6(ctx, ctx->uind, ctx->fld6));
   k_init_rsd<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->fld6, ctx->efield, ctx->udir, ctx->uind, ctx->rsd, guess);
   if (A.sparse)
      T9_CHECK(launch_precond_sparse(ctx, ctx->rsd, ctx->zrsd));
   k_precond_dot<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->rsd, ctx->zrsd, ctx->conj, ctx->red, 1);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

static int induce_once(Context* ctx)
{
   const VecArgs A = vec_args(ctx);
   T9_CHECK(pcg_start(ctx, A));
   const int politer = std::max(1, ctx->cfg.politer);
   for (int it = 0; it < politer; ++it) {
      T9_CHECK(pcg_body(ctx, A));
      T9_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->status, sizeof(int) * ST_NSTAT, cudaMemcpyDeviceToHost,
         ctx->stream));
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
      if (ctx->h_status[ST_DONE])
         break;
   }
   T9_CUDA(cudaMemcpyAsync(ctx->h_scal, ctx->scal, sizeof(double) * S_COEF, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return T9GB_OK;
}

int induce_sorted(Context* ctx)
{
   int redo = 0;
   T9_CHECK(induce_once(ctx));
   T9_CHECK(check_list_overflow(ctx, &redo));
   if (redo)
      T9_CHECK(induce_once(ctx));
   // predictor history (ulspredSave, src/amoeba/induce.cpp:29-63)
   if (ctx->cfg.predictor == 1) {
      float* dst = ctx->aspc_hist + (size_t)(ctx->nualt % 16) * 6 * ctx->npad;
      k_copy<<<grid_for(6 * ctx->npad, 256), 256, 0, ctx->stream>>>(6 * ctx->npad, ctx->uind, dst);
      T9_CUDA(cudaGetLastError());
      ctx->nualt += 1;
      if (ctx->nualt > 32)
         ctx->nualt -= 16;
   }
   prof_collect(ctx);
   ctx->last_iter = ctx->h_status[ST_ITER];
   ctx->last_eps = ctx->h_scal[S_EPS];
   ctx->last_status = ctx->h_status[ST_STATUS];
   return ctx->last_status;
}

// ---------------------------------------------------------------------------
// public field entry points (sorted internally, caller order at the boundary)

template <class F>
static int with_list(Context* ctx, F&& body)
{
   for (int attempt = 0; attempt < 2; ++attempt) {
      T9_CHECK(ensure_list(ctx));
      T9_CHECK(body());
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
      int redo = 0;
      T9_CHECK(check_list_overflow(ctx, &redo));
      if (!redo)
         return T9GB_OK;
   }
   return T9GB_OK;
}

int public_dfield(Context* ctx, float* field, float* fieldp)
{
   return with_list(ctx, [&]() {
      T9_CHECK(dfield6(ctx, ctx->tmp6));
      return scatter_from_sorted3(ctx, ctx->tmp6, field, fieldp);
   });
}

int public_ufield(Context* ctx, const float* uind, const float* uinp, float* field, float* fieldp)
{
   return with_list(ctx, [&]() {
      T9_CHECK(gather_to_sorted3(ctx, uind, uinp, ctx->tmp6));
      T9_CHECK(ufield6(ctx, ctx->tmp6, ctx->vec));
      return scatter_from_sorted3(ctx, ctx->vec, field, fieldp);
   });
}

int public_precond(Context* ctx, const float* rsd, const float* rsdp, float* zrsd, float* zrsdp)
{
   return with_list(ctx, [&]() {
      T9_CHECK(gather_to_sorted3(ctx, rsd, rsdp, ctx->tmp6));
      T9_CHECK(launch_precond_sparse(ctx, ctx->tmp6, ctx->vec));
      return scatter_from_sorted3(ctx, ctx->vec, zrsd, zrsdp);
   });
}

}  // namespace t9gb
