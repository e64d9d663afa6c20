// Learned initial guess of the induced dipoles.
//
// Per slot s and per dipole set (d, p) the network (mlp.cu) maps 32
// rotation-invariant features (pair.cu, k_learn_features) to a correction of
// the direct guess, expressed in the atom's local multipole frame F and in
// field units:
//     u_guess = alpha E + alpha F^T y tscale.
// Training targets come from the converged PCG dipoles of the same solve,
//     t = F (u - alpha E) / (alpha tscale),
// so the network learns the frame-resolved mutual field -T u.  Every piece
// is a device kernel on the context's stream, so guess, fallback test and
// training are part of the induce() CUDA graph.
//
// Fallback: the solve computes the starting residual of both the plain guess
// (the ASPC predictor when its history is full, else alpha E) and the learned
// guess and, separately for d and p, starts from the one with the smaller
// r.r; a tie keeps the plain guess.  The PCG then iterates to the same RMS
// threshold as without the network.
//
// The reference has no learned component: its guesses are alpha E
// (src/cu/amoeba/induce.cu, pcgUdirV2) and the ASPC/GEAR/LSQR predictors
// (src/amoeba/induce.cpp:29-69).
#include <cmath>

#include "common.cuh"
#include "reduce.cuh"

namespace t9gb {

constexpr int LB = 256;  // block size (sum_slots needs 256)
constexpr int F_MEAN = 0, F_ISTD = 32, F_TSCALE = 64;

// per-column mean and 1/std of the raw features over the rows of real atoms;
// runs once (bit 0 of ST_LREADY), one block per column
__global__ void k_feature_stats(int npad, const float* __restrict__ xf, const float* __restrict__ polar,
   float* __restrict__ fstat, int* __restrict__ state)
{
   __shared__ double sh[40];
   if (state[ST_LREADY] & 1) {
      // fixed before this solve: the feature kernel has normalised
      if (blockIdx.x == 0 && threadIdx.x == 0)
         state[ST_LREADY] &= ~8;
      return;
   }
   const int c = blockIdx.x;
   double s1 = 0, s2 = 0, cnt = 0;
   for (int r = threadIdx.x; r < 2 * npad; r += blockDim.x) {
      if (polar[r % npad] == 0.f)
         continue;
      const double v = xf[(size_t)r * 32 + c];
      s1 += v;
      s2 += v * v;
      cnt += 1;
   }
   s1 = block_sum(s1, sh);
   s2 = block_sum(s2, sh);
   cnt = block_sum(cnt, sh);
   if (threadIdx.x == 0) {
      const double mean = cnt > 0 ? s1 / cnt : 0.0;
      const double var = cnt > 0 ? fmax(s2 / cnt - mean * mean, 0.0) : 0.0;
      const double sd = sqrt(var);
      fstat[F_MEAN + c] = (float)mean;
      fstat[F_ISTD + c] = sd > 1e-6 * (fabs(mean) + 1e-3) ? (float)(1.0 / sd) : 0.f;
   }
   if (last_block(state + ST_TICKET1) && threadIdx.x == 0)
      state[ST_LREADY] |= 1 | 8;  // bit 3: k_normalize runs in this solve
}

// BF16 network input: (x - mean) / std, zero rows for padding slots.  Only
// in the solve that fixed the statistics (bit 3); afterwards the feature
// kernel writes it.
__global__ void k_normalize(int npad, const float* __restrict__ xf, const float* __restrict__ polar,
   const float* __restrict__ fstat, const int* __restrict__ state, __nv_bfloat16* __restrict__ x)
{
   if (!(state[ST_LREADY] & 8))
      return;
   const int total = 2 * npad * 32;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
      const int r = e / 32, c = e % 32;
      float v = 0.f;
      if (polar[r % npad] != 0.f)
         v = (xf[e] - fstat[F_MEAN + c]) * fstat[F_ISTD + c];
      x[e] = __float2bfloat16(v);
   }
}

// u_guess = udir + alpha F^T y tscale (rows [npad][8], components 0-5);
// set_choice: record that both systems start from it
__global__ void k_learned_guess(int npad, const float* __restrict__ udir, const float* __restrict__ y,
   const float* __restrict__ frame, const float* __restrict__ polar, const float* __restrict__ fstat,
   int* __restrict__ state, float* __restrict__ ug, int set_choice)
{
   const float ts = (state[ST_LREADY] & 2) ? fstat[F_TSCALE] : 0.f;
   if (set_choice && blockIdx.x == 0 && threadIdx.x == 0)
      state[ST_LCHOICE] = 3;
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      const float* F = frame + 9 * s;
      const float a = polar[s] * ts;
      for (int sys = 0; sys < 2; ++sys) {
         const float* yr = y + (size_t)(sys * npad + s) * MLP_OUT_PAD;
         for (int c = 0; c < 3; ++c) {
            const float v = F[c] * yr[0] + F[3 + c] * yr[1] + F[6 + c] * yr[2];
            ug[8 * s + 3 * sys + c] = udir[8 * s + 3 * sys + c] + a * v;
         }
      }
   }
}

// r.r of the plain residual (rsd) and of the learned one
// rL = (udir - uL)/alpha + fldL; the last block picks per d/p system
__global__ void k_resid_cmp(int ne, const float* __restrict__ polar, const float* __restrict__ polinv,
   const float* __restrict__ udir, const float* __restrict__ uL, const float* __restrict__ fldL,
   const float* __restrict__ rsd, double* __restrict__ red, double* __restrict__ scal, int* __restrict__ state)
{
   __shared__ double sh[64];
   double pd = 0, pp = 0, ld = 0, lp = 0;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;
      const float r0 = rsd[x];
      float r1 = (udir[x] - uL[x]) * polinv[s] + fldL[x];
      if (polar[s] == 0.f)
         r1 = 0.f;
      if (e - 6 * s < 3) {
         pd += (double)r0 * r0;
         ld += (double)r1 * r1;
      } else {
         pp += (double)r0 * r0;
         lp += (double)r1 * r1;
      }
   }
   const double pv[4] = {pd, pp, ld, lp};
   store_partials<4>(red, 0, pv, sh);
   if (!last_block(state + ST_TICKET0))
      return;
   double tot[4];
   sum_slots(red, 0, 4, gridDim.x, sh, tot);
   if (threadIdx.x == 0) {
      // a learned guess whose field left the grid's fixed-point range has no
      // valid residual: the plain start is kept
      const bool out = state[ST_RANGE_L] != 0;
      state[ST_RANGE_L] = 0;
      scal[S_L_PLAIN_D] = tot[0];
      scal[S_L_PLAIN_P] = tot[1];
      scal[S_L_LEARN_D] = out ? INFINITY : tot[2];
      scal[S_L_LEARN_P] = out ? INFINITY : tot[3];
      state[ST_LCHOICE] = out ? 0 : (tot[2] < tot[0] ? 1 : 0) | (tot[3] < tot[1] ? 2 : 0);
   }
}

// start the chosen systems from the learned guess
__global__ void k_resid_pick(int ne, const float* __restrict__ polar, const float* __restrict__ polinv,
   const float* __restrict__ udir, const float* __restrict__ uL, const float* __restrict__ fldL,
   float* __restrict__ uind, float* __restrict__ rsd, const int* __restrict__ state)
{
   const int choice = state[ST_LCHOICE];
   if (choice == 0)
      return;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;
      const int sys = e - 6 * s < 3 ? 1 : 2;
      if (!(choice & sys))
         continue;
      float r1 = (udir[x] - uL[x]) * polinv[s] + fldL[x];
      if (polar[s] == 0.f)
         r1 = 0.f;
      uind[x] = uL[x];
      rsd[x] = r1;
   }
}

// target scale: RMS over real atoms and both systems of F (u - udir) / alpha;
// runs once (bit 1 of ST_LREADY), one block
__global__ void k_target_scale(int npad, const float* __restrict__ uind, const float* __restrict__ udir,
   const float* __restrict__ frame, const float* __restrict__ polar, float* __restrict__ fstat,
   int* __restrict__ state)
{
   __shared__ double sh[40];
   if (state[ST_LREADY] & 2)
      return;
   double s2 = 0, cnt = 0;
   for (int s = threadIdx.x; s < npad; s += blockDim.x) {
      const float a = polar[s];
      if (a == 0.f)
         continue;
      for (int k = 0; k < 6; ++k) {
         const double v = (uind[8 * s + k] - udir[8 * s + k]) / a;
         s2 += v * v;  // a rotation keeps the norm
      }
      cnt += 6;
   }
   s2 = block_sum(s2, sh);
   cnt = block_sum(cnt, sh);
   if (threadIdx.x == 0) {
      const double rms = cnt > 0 ? sqrt(s2 / cnt) : 0.0;
      fstat[F_TSCALE] = rms > 0 ? (float)rms : 1.f;
      state[ST_LREADY] |= 2;
   }
}

// t[r] = F (u - udir) / (alpha tscale) for rows r = sys * npad + s
__global__ void k_targets(int npad, const float* __restrict__ uind, const float* __restrict__ udir,
   const float* __restrict__ frame, const float* __restrict__ polar, const float* __restrict__ fstat,
   float* __restrict__ t)
{
   const float its = 1.f / fstat[F_TSCALE];
   for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < 2 * npad; r += gridDim.x * blockDim.x) {
      const int s = r % npad, o = 3 * (r / npad);
      const float a = polar[s];
      float v[3] = {0.f, 0.f, 0.f};
      if (a != 0.f) {
         const float w = its / a;
         for (int c = 0; c < 3; ++c)
            v[c] = (uind[8 * s + o + c] - udir[8 * s + o + c]) * w;
      }
      const float* F = frame + 9 * s;
      for (int k = 0; k < 3; ++k)
         t[(size_t)r * 3 + k] = F[3 * k] * v[0] + F[3 * k + 1] * v[1] + F[3 * k + 2] * v[2];
   }
}

__global__ void k_store_loss(const double* __restrict__ loss, double norm, double* __restrict__ scal)
{
   scal[S_L_LOSS] = *loss * norm;
}

// ---------------------------------------------------------------------------

int learn_setup(Context* ctx)
{
   if (ctx->xf)
      return T9GB_OK;
   const size_t rows = 2 * (size_t)ctx->npad;
   T9_CUDA(cudaMalloc(&ctx->xf, sizeof(float) * rows * 32));
   T9_CUDA(cudaMemset(ctx->xf, 0, sizeof(float) * rows * 32));
   T9_CUDA(cudaMalloc(&ctx->fstat, sizeof(float) * 72));
   T9_CUDA(cudaMemset(ctx->fstat, 0, sizeof(float) * 72));
   T9_CUDA(cudaDeviceSynchronize());
   T9_CHECK(mlp_alloc(ctx, (int)rows, ctx->learn_seed));
   return T9GB_OK;
}

void learn_free(Context* ctx)
{
   if (ctx->xf)
      cudaFree(ctx->xf);
   if (ctx->fstat)
      cudaFree(ctx->fstat);
   ctx->xf = nullptr;
   ctx->fstat = nullptr;
   mlp_free(ctx);
}

// fresh weights from `seed`, statistics and moments cleared (buffers kept,
// so a captured graph stays valid)
int learn_reset(Context* ctx, unsigned seed)
{
   ctx->learn_seed = seed;
   T9_CHECK(learn_setup(ctx));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   T9_CHECK(mlp_alloc(ctx, 2 * ctx->npad, seed));
   T9_CUDA(cudaMemsetAsync(ctx->status + ST_LREADY, 0, sizeof(int), ctx->stream));
   T9_CUDA(cudaMemsetAsync(ctx->status + ST_LCHOICE, 0, sizeof(int), ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return T9GB_OK;
}

// features of the current solve (efield, udir), statistics, forward pass
// (need_y: the guess reads the outputs; the mma.sync training path reads
// the activations; the tcgen05 training pass recomputes both)
int learn_forward(Context* ctx, bool need_y)
{
   const int npad = ctx->npad;
   T9_CHECK(launch_learn_features(ctx, ctx->efield, ctx->udir, ctx->xf, ctx->fstat, ctx->mlp.x));
   k_feature_stats<<<32, LB, 0, ctx->stream>>>(npad, ctx->xf, ctx->spolar, ctx->fstat, ctx->status);
   // grid-stride: usually every block returns at once
   k_normalize<<<std::min(512, grid_for(2LL * npad * 32, LB)), LB, 0, ctx->stream>>>(npad, ctx->xf, ctx->spolar,
      ctx->fstat, ctx->status, ctx->mlp.x);
   T9_CUDA(cudaGetLastError());
   if (need_y || (!ctx->mlp_tc && (ctx->learn_mode & 1)))
      return mlp_forward(ctx, 2 * npad);
   return T9GB_OK;
}

int learn_guess(Context* ctx, float* ug8, int set_choice)
{
   k_learned_guess<<<grid_for(ctx->npad, LB), LB, 0, ctx->stream>>>(ctx->npad, ctx->udir, ctx->mlp.y, ctx->sframe,
      ctx->spolar, ctx->fstat, ctx->status, ug8, set_choice);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int learn_pick(Context* ctx, const float* ug8, const float* fld8)
{
   const int ne = 6 * ctx->npad;
   const int nb = std::min(RED_MAX, grid_for(ne, LB));
   k_resid_cmp<<<nb, LB, 0, ctx->stream>>>(ne, ctx->spolar, ctx->spolinv, ctx->udir, ug8, fld8, ctx->rsd, ctx->red,
      ctx->scal, ctx->status);
   k_resid_pick<<<nb, LB, 0, ctx->stream>>>(ne, ctx->spolar, ctx->spolinv, ctx->udir, ug8, fld8, ctx->uind, ctx->rsd,
      ctx->status);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// one AdamW step on the converged dipoles of this solve (after learn_forward)
int learn_train(Context* ctx)
{
   const int npad = ctx->npad;
   k_target_scale<<<1, LB, 0, ctx->stream>>>(npad, ctx->uind, ctx->udir, ctx->sframe, ctx->spolar, ctx->fstat,
      ctx->status);
   k_targets<<<grid_for(2 * npad, LB), LB, 0, ctx->stream>>>(npad, ctx->uind, ctx->udir, ctx->sframe, ctx->spolar,
      ctx->fstat, ctx->mlp.t);
   T9_CUDA(cudaGetLastError());
   const double norm = 1.0 / (6.0 * std::max(1, ctx->n));
   if (ctx->mlp_tc)
      return mlp_train_step_tc(ctx, 2 * npad, ctx->spolar, npad, ctx->learn_lr, ctx->learn_wd, ctx->scal + S_L_LOSS,
         norm);
   T9_CHECK(mlp_backward(ctx, 2 * npad, ctx->spolar, npad));
   k_store_loss<<<1, 1, 0, ctx->stream>>>(ctx->mlp.loss, norm, ctx->scal);
   T9_CHECK(mlp_adamw(ctx, ctx->learn_lr, ctx->learn_wd));
   return T9GB_OK;
}

// raw features [2n][32] in caller order (d rows, then p rows)
__global__ void k_features_out(int n, int npad, const int* __restrict__ iperm, const float* __restrict__ xf,
   float* __restrict__ out)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 2 * n * 32; e += gridDim.x * blockDim.x) {
      const int r = e / 32, c = e % 32;
      const int sys = r / n, i = r % n;
      out[e] = xf[(size_t)(sys * npad + iperm[i]) * 32 + c];
   }
}

int learn_features_out(Context* ctx, float* out_dev)
{
   k_features_out<<<grid_for(2LL * ctx->n * 32, LB), LB, 0, ctx->stream>>>(ctx->n, ctx->npad, ctx->iperm, ctx->xf,
      out_dev);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

}  // namespace t9gb
