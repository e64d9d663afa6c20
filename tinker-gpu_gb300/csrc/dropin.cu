// Entry points that let the C++ drop-in layer (t9gb_tinker.cpp) keep the
// reference's data contracts: coordinates from its structure-of-arrays
// `x, y, z` device arrays, the diagonal preconditioner on caller-order
// vectors, and gradients in its fixed-point `grad_prec` form.
#include "common.cuh"

namespace t9gb {

__global__ void k_xyz_from_soa(int n, const float* __restrict__ x, const float* __restrict__ y,
   const float* __restrict__ z, float* __restrict__ xyz)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n)
      return;
   xyz[3 * i] = x[i];
   xyz[3 * i + 1] = y[i];
   xyz[3 * i + 2] = z[i];
}

// z = alpha r, caller order (reference: diagPrecond_cu1,
// src/cu/diagprecond.cu:5-28); rsdp / zrsdp may be null together.
__global__ void k_diag_precond(int n, const int* __restrict__ iperm, const float* __restrict__ spolar,
   const float* __restrict__ rsd, const float* __restrict__ rsdp, float* __restrict__ zrsd,
   float* __restrict__ zrsdp)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n)
      return;
   const float a = spolar[iperm[i]];
   for (int d = 0; d < 3; ++d)
      zrsd[3 * i + d] = a * rsd[3 * i + d];
   if (rsdp)
      for (int d = 0; d < 3; ++d)
         zrsdp[3 * i + d] = a * rsdp[3 * i + d];
}

// Float gradient [n][3] -> fixed point at 2^32 per unit, truncated toward
// zero through a signed 64-bit integer, the conversion of the reference's
// floatTo<fixed> / atomic_add(T, fixed*) (include/syntax/cu/adddef.h:36-71).
// One thread per atom and component writes its own word, so the result does
// not depend on scheduling; accumulate adds to the words like sumGradient
// (src/cu/egvop.cu:6-14).
__global__ void k_grad_fixed(int n, const float* __restrict__ g, int accumulate, unsigned long long* __restrict__ gx,
   unsigned long long* __restrict__ gy, unsigned long long* __restrict__ gz)
{
   const int t = blockIdx.x * blockDim.x + threadIdx.x;
   if (t >= 3 * n)
      return;
   const int i = t / 3, d = t - 3 * i;
   const unsigned long long v = g ? (unsigned long long)(long long)((double)g[t] * 4294967296.0) : 0ull;
   unsigned long long* out = d == 0 ? gx : (d == 1 ? gy : gz);
   out[i] = accumulate ? out[i] + v : v;
}

}  // namespace t9gb

using namespace t9gb;

extern "C" {

int t9gb_set_xyz_soa_device(t9gb_context* h, const float* x, const float* y, const float* z)
{
   if (!h || !x || !y || !z)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   k_xyz_from_soa<<<grid_for(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, x, y, z, ctx->xyz);
   T9_CUDA(cudaGetLastError());
   ctx->have_xyz = true;
   if (ctx->have_order)
      T9_CHECK(scatter_positions(ctx));
   return T9GB_OK;
}

int t9gb_diag_precond_apply(t9gb_context* h, const float* rsd, const float* rsdp, float* zrsd, float* zrsdp)
{
   if (!h || !rsd || !zrsd || (!rsdp) != (!zrsdp))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_order)
      return T9GB_NOT_READY;
   k_diag_precond<<<grid_for(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, ctx->iperm, ctx->spolar, rsd, rsdp, zrsd,
      zrsdp);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int t9gb_gradient_fixed(t9gb_context* h, const float* grad_device, int accumulate, unsigned long long* gx,
   unsigned long long* gy, unsigned long long* gz)
{
   if (!h || !gx || !gy || !gz || (!grad_device && accumulate))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   k_grad_fixed<<<grid_for(3LL * ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, grad_device, accumulate ? 1 : 0, gx,
      gy, gz);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

}  // extern "C"
