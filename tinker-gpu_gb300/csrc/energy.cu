// Energies that consume the multipoles and the converged dipoles, with
// deterministic FP64 reductions.
//
//  - t9gb_empole_energy: permanent-multipole energy, real + reciprocal + self
//    (empole(calc::energy), src/amoeba/empole.cpp:81-138); the one-body
//    "self" part also holds the external-field term when a field is set;
//  - t9gb_epolar_energy: polarization energy by the dot product
//    -1/2 f sum_i u_d,i . E_p,i (epolar0DotProd, src/cu/amoeba/epolar.cu:14-30);
//  - t9gb_empole / t9gb_epolar / t9gb_emplar: energy and gradient with the
//    reference's calc flags (include/tool/rcman.h:105-155), forces from
//    force.cu.
#include "common.cuh"
#include "reduce.cuh"

namespace t9gb {

// Fixed-order FP64 row sums spread over SUM_PARTS blocks per row (an FP64 add
// on this GPU issues at a small fraction of the FP32 rate, so one SM per row
// is slow): block (p, r) sums its segment of row r into part[r][p], and the
// last block of the launch adds each row's parts in order into out[r].

template <class T>
__global__ void __launch_bounds__(256) k_sum_rows_t(int n, int stride, const T* __restrict__ a,
   double* __restrict__ part, double* __restrict__ out, int* __restrict__ ticket)
{
   __shared__ double sh[8];
   const int r = blockIdx.y, p = blockIdx.x;
   const T* row = a + (size_t)r * stride;
   const int seg = (n + SUM_PARTS - 1) / SUM_PARTS, b = p * seg, e = min(n, b + seg);
   double v = 0;
   for (int i = b + threadIdx.x; i < e; i += blockDim.x)
      v += (double)row[i];
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
      v += __shfl_down_sync(0xffffffffu, v, o);
   if ((threadIdx.x & 31) == 0)
      sh[threadIdx.x >> 5] = v;
   __syncthreads();
   if (threadIdx.x == 0) {
      double t = 0;
      for (int w = 0; w < (int)(blockDim.x >> 5); ++w)
         t += sh[w];
      part[(size_t)r * SUM_PARTS + p] = t;
   }
   // the last block of the launch combines every row's parts
   __shared__ bool last;
   __threadfence();
   __syncthreads();
   if (threadIdx.x == 0)
      last = atomicAdd(reinterpret_cast<unsigned*>(ticket), 1u) == gridDim.x * gridDim.y - 1;
   __syncthreads();
   if (!last)
      return;
   __threadfence();
   for (int rr = threadIdx.x; rr < (int)gridDim.y; rr += blockDim.x) {
      double t = 0;
      for (int q = 0; q < SUM_PARTS; ++q)
         t += part[(size_t)rr * SUM_PARTS + q];
      out[rr] = t;
   }
   if (threadIdx.x == 0)
      *ticket = 0;
}

// out[0..rows) = the fixed-order sums of rows of n entries (stride apart)
template <class T>
static int sum_rows_launch(Context* ctx, int rows, int n, int stride, const T* a, double* out)
{
   if (rows < 1 || rows > SUM_ROWS_MAX)
      return T9GB_BAD_ARG;
   k_sum_rows_t<T><<<dim3(SUM_PARTS, rows), 256, 0, ctx->stream>>>(n, stride, a, ctx->sum_part, out,
      ctx->status + ST_TICKET_SUM);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// e[s] = -1/2 f alpha_s^-1 (u_d . udir_p)
__global__ void k_epolar_dot(int npad, double f, const float* __restrict__ uind, const float* __restrict__ udir,
   const float* __restrict__ polinv, double* __restrict__ e)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      const float* u = uind + 8 * s;
      const float* p = udir + 8 * s + 3;
      e[s] = -0.5 * f * (double)polinv[s] * ((double)u[0] * p[0] + (double)u[1] * p[1] + (double)u[2] * p[2]);
   }
}

}  // namespace t9gb

using namespace t9gb;


extern "C" int t9gb_empole_energy(t9gb_context* h, double* energy, double* parts)
{
   if (!h || !energy)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   for (int attempt = 0; attempt < 2; ++attempt) {
      T9_CHECK(ensure_list(ctx));
      T9_CUDA(cudaMemsetAsync(ctx->e_atom, 0, sizeof(double) * 3 * ctx->npad, ctx->stream));
      T9_CHECK(launch_empole_real(ctx, ctx->e_atom));
      T9_CHECK(launch_empole_recip(ctx, ctx->e_atom + ctx->npad));
      T9_CHECK(launch_extfield_mpole(ctx, false, false));
      T9_CHECK(sum_rows_launch(ctx, 3, ctx->npad, ctx->npad, ctx->e_atom, ctx->scal + 32));
      T9_CUDA(cudaMemcpyAsync(ctx->h_scal + 32, ctx->scal + 32, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->stream));
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
      int redo = 0;
      T9_CHECK(check_list_overflow(ctx, &redo));
      if (!redo)
         break;
   }
   const double* v = ctx->h_scal + 32;
   *energy = v[0] + v[1] + v[2];
   if (parts) {
      parts[0] = v[0];
      parts[1] = v[1];
      parts[2] = v[2];
   }
   return T9GB_OK;
}

extern "C" int t9gb_epolar_energy(t9gb_context* h, double* energy)
{
   if (!h || !energy)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   k_epolar_dot<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, ctx->cfg.electric, ctx->uind, ctx->udir,
      ctx->spolinv, ctx->e_atom);
   T9_CHECK(sum_rows_launch(ctx, 1, ctx->npad, ctx->npad, ctx->e_atom, ctx->scal + 36));
   T9_CUDA(cudaMemcpyAsync(ctx->h_scal + 36, ctx->scal + 36, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   *energy = ctx->h_scal[36];
   return T9GB_OK;
}

namespace t9gb {

// fixed-order sum of nrows FP64 rows of npad per-slot terms
int sum_rows_d(Context* ctx, const double* rows, int nrows, double* out)
{
   T9_CHECK(sum_rows_launch(ctx, nrows, ctx->npad, ctx->npad, rows, ctx->scal + 52));
   double v[8];
   T9_CUDA(cudaMemcpyAsync(v, ctx->scal + 52, sizeof(double) * nrows, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   double t = 0;
   for (int r = 0; r < nrows; ++r)
      t += v[r];
   *out = t;
   return T9GB_OK;
}

// nblocks blocks of 9 FP32 virial rows [9][npad], summed and symmetrised
int sum_rows_virial(Context* ctx, const float* rows, int nblocks, double* virial)
{
   T9_CHECK(sum_rows_launch(ctx, 9 * nblocks, ctx->npad, ctx->npad, rows, ctx->vsum));
   double v[27];
   T9_CUDA(cudaMemcpyAsync(v, ctx->vsum, sizeof(double) * 9 * nblocks, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   double W[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
   for (int b = 0; b < nblocks; ++b)
      for (int c = 0; c < 9; ++c)
         W[c] += v[9 * b + c];
   for (int a = 0; a < 3; ++a)
      for (int c = 0; c < 3; ++c)
         virial[3 * a + c] = 0.5 * (W[3 * a + c] + W[3 * c + a]);
   return T9GB_OK;
}

static int sum_empole(Context* ctx, double* energy)
{
   T9_CHECK(sum_rows_launch(ctx, 3, ctx->npad, ctx->npad, ctx->e_atom, ctx->scal + 32));
   T9_CUDA(cudaMemcpyAsync(ctx->h_scal + 32, ctx->scal + 32, sizeof(double) * 3, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   *energy = ctx->h_scal[32] + ctx->h_scal[33] + ctx->h_scal[34];
   return T9GB_OK;
}

static int check_vers(Context* ctx, int vers, double* energy, float* grad, double* virial)
{
   if ((vers & T9GB_CALC_ENERGY) && !energy)
      return T9GB_BAD_ARG;
   if ((vers & T9GB_CALC_GRAD) && !grad)
      return T9GB_BAD_ARG;
   if ((vers & T9GB_CALC_VIRIAL) && !virial)
      return T9GB_BAD_ARG;
   if (!(vers & (T9GB_CALC_ENERGY | T9GB_CALC_GRAD | T9GB_CALC_VIRIAL)))
      return T9GB_BAD_ARG;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   return T9GB_OK;
}

// mpole / polar terms on the current coordinates and rotated multipoles
// virial: sum of the per-slot rows (real, frame, reciprocal transform) and
// the k-space sums, symmetrised; row-major 3 x 3
static int sum_virial(Context* ctx, double* virial)
{
   T9_CHECK(sum_rows_launch(ctx, 27, ctx->npad, ctx->npad, ctx->wvir, ctx->vsum));
   double v[27], k[12];
   T9_CUDA(cudaMemcpyAsync(v, ctx->vsum, sizeof(double) * 27, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaMemcpyAsync(k, ctx->scal + 40, sizeof(double) * 12, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   if (!ctx->cfg.use_ewald)
      for (double& x : k)
         x = 0;
   const int ab[6][2] = {{0, 0}, {1, 1}, {2, 2}, {0, 1}, {0, 2}, {1, 2}};
   double W[3][3];
   for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
         W[a][b] = v[3 * a + b] + v[9 + 3 * a + b] + v[18 + 3 * a + b];
   // the influence-function sums are symmetric: component ab is also ba
   for (int c = 0; c < 6; ++c) {
      const double kv = k[c] + k[6 + c];
      W[ab[c][0]][ab[c][1]] += kv;
      if (c >= 3)
         W[ab[c][1]][ab[c][0]] += kv;
   }
   for (int a = 0; a < 3; ++a)
      for (int b = 0; b < 3; ++b)
         virial[3 * a + b] = 0.5 * (W[a][b] + W[b][a]);
   return T9GB_OK;
}

static int elec_terms(Context* ctx, bool mpole, bool polar, int vers, double* energy, float* grad, double* virial,
   const std::function<int()>* beside = nullptr)
{
   double e = 0;
   if (polar) {
      int rc = induce_sorted(ctx);
      if (rc != T9GB_OK)
         return rc;
   }
   bool beside_done = false;
   for (int attempt = 0; attempt < 2; ++attempt) {
      // a list refreshed here needs its capacity checked; one already checked
      // (after the solve above, or an earlier call) does not, and the gradient
      // then stays in stream order without a synchronisation
      const bool fresh = ctx->list_stale || ctx->list_need_build;
      T9_CHECK(ensure_list(ctx));
      // work that reads the list starts once the list is final: here when it
      // was current already, else after the capacity check below
      if (beside && !beside_done && !fresh) {
         T9_CHECK((*beside)());
         beside_done = true;
      }
      T9_CUDA(cudaMemsetAsync(ctx->e_atom, 0, sizeof(double) * 3 * ctx->npad, ctx->stream));
      if (vers & (T9GB_CALC_GRAD | T9GB_CALC_VIRIAL)) {
         T9_CHECK(elec_forces(ctx, mpole, polar, (vers & T9GB_CALC_GRAD) ? grad : nullptr,
            (vers & T9GB_CALC_VIRIAL) != 0));
      } else if (mpole) {
         T9_CHECK(launch_empole_real(ctx, ctx->e_atom));
         T9_CHECK(launch_empole_recip(ctx, ctx->e_atom + ctx->npad));
         T9_CHECK(launch_extfield_mpole(ctx, false, false));
      }
      if (!fresh)
         break;
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
      int redo = 0;
      T9_CHECK(check_list_overflow(ctx, &redo));
      if (!redo)
         break;
   }
   if (beside && !beside_done)
      T9_CHECK((*beside)());
   if (vers & T9GB_CALC_ENERGY) {
      if (mpole)
         T9_CHECK(sum_empole(ctx, &e));
      if (polar) {
         k_epolar_dot<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, ctx->cfg.electric, ctx->uind,
            ctx->udir, ctx->spolinv, ctx->e_atom);
         T9_CHECK(sum_rows_launch(ctx, 1, ctx->npad, ctx->npad, ctx->e_atom, ctx->scal + 36));
         T9_CUDA(cudaMemcpyAsync(ctx->h_scal + 36, ctx->scal + 36, sizeof(double), cudaMemcpyDeviceToHost,
            ctx->stream));
         T9_CUDA(cudaStreamSynchronize(ctx->stream));
         e += ctx->h_scal[36];
      }
      *energy = e;
   }
   if (vers & T9GB_CALC_VIRIAL)
      T9_CHECK(sum_virial(ctx, virial));
   return T9GB_OK;
}

// The MD step's gradient: the forces (and the beside work) are queued right
// behind the induce graph, before the solve's status synchronisation, so the
// device does not wait for the host between the solve and the forces; the
// same kernels in the same stream order as elec_terms.  When the solve had to
// be repeated (a list or range retry) the queued work used the discarded
// solve: reset() clears what the beside work accumulates and the forces are
// queued again on the final solve and list.
int emplar_grad_beside(Context* ctx, float* grad, const std::function<int()>& beside,
   const std::function<int()>& reset)
{
   if (!ctx->use_graph || ctx->prof.on)
      return elec_terms(ctx, true, true, T9GB_CALC_GRAD, nullptr, grad, nullptr, &beside);
   const std::function<int()> forces = [&]() -> int {
      T9_CHECK(beside());
      T9_CUDA(cudaMemsetAsync(ctx->e_atom, 0, sizeof(double) * 3 * ctx->npad, ctx->stream));
      return elec_forces(ctx, true, true, grad, false);
   };
   ctx->after_launch = &forces;
   ctx->after_done = false;
   const int rc = induce_sorted(ctx);
   const bool queued = ctx->after_done, redone = ctx->induce_redone;
   ctx->after_launch = nullptr;
   ctx->after_done = false;
   if (rc != T9GB_OK)
      return rc;
   if (queued && !redone)
      return T9GB_OK;
   if (queued)
      T9_CHECK(reset());
   T9_CHECK(ensure_list(ctx));
   return forces();
}

}  // namespace t9gb

extern "C" int t9gb_energy_components(t9gb_context* h, double* parts)
{
   if (!h || !parts)
      return T9GB_BAD_ARG;
   for (int c = 0; c < 4; ++c)
      parts[c] = h->c.h_scal[32 + c + (c == 3 ? 1 : 0)];
   return T9GB_OK;
}

extern "C" int t9gb_empole(t9gb_context* h, int vers, double* energy, float* grad, double* virial)
{
   if (!h)
      return T9GB_BAD_ARG;
   T9_CHECK(check_vers(&h->c, vers, energy, grad, virial));
   return elec_terms(&h->c, true, false, vers, energy, grad, virial);
}

extern "C" int t9gb_epolar(t9gb_context* h, int vers, double* energy, float* grad, double* virial)
{
   if (!h)
      return T9GB_BAD_ARG;
   T9_CHECK(check_vers(&h->c, vers, energy, grad, virial));
   return elec_terms(&h->c, false, true, vers, energy, grad, virial);
}

extern "C" int t9gb_emplar(t9gb_context* h, int vers, double* energy, float* grad, double* virial)
{
   if (!h)
      return T9GB_BAD_ARG;
   T9_CHECK(check_vers(&h->c, vers, energy, grad, virial));
   return elec_terms(&h->c, true, true, vers, energy, grad, virial);
}
