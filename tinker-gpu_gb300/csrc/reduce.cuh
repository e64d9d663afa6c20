// Device scalars, status words and the fixed-order FP64 reductions shared by
// the PCG (pcg.cu) and the learned guess (learn.cu).
#pragma once
#include "common.cuh"

namespace t9gb {

// device doubles (ctx->scal) and ints (ctx->status)
// S_L_*: learned guess -- r.r of the plain and the learned starting residual
// (d, p) and the last training loss
enum { S_SUM_D = 0, S_SUM_P, S_A_D, S_A_P, S_B_D, S_B_P, S_EPS, S_L_PLAIN_D = 8, S_L_PLAIN_P, S_L_LEARN_D,
   S_L_LEARN_P, S_L_LOSS, S_NSCAL = 16 };
// ST_LCHOICE: bit 0 / 1 set when the d / p solve started from the learned
// guess; ST_LREADY: bit 0 feature statistics, bit 1 target scale fixed
enum { ST_ITER = 0, ST_DONE, ST_STATUS, ST_NUALT, ST_TICKET0, ST_TICKET1, ST_LCHOICE, ST_LREADY, ST_NSTAT = 8 };
enum { R_PAP_D = 0, R_PAP_P, R_RZ_D, R_RZ_P, R_RR_D, R_RR_P };

static __device__ __forceinline__ double block_sum(double v, double* sh)
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

// Fixed-order sums of `ns` (<= 4) consecutive partial slots, computed
// together: 64 threads per slot stride through the nb partials, then a fixed
// shuffle tree and one combine (blockDim must be 256).  Returns the sums in
// out[0..ns) of every thread.
static __device__ __forceinline__ void sum_slots(const double* red, int first, int ns, int nb, double* sh, double* out)
{
   const int slot = threadIdx.x >> 6, sub = threadIdx.x & 63;
   double v = 0;
   if (slot < ns)
      for (int i = sub; i < nb; i += 64)
         v += red[(first + slot) * RED_MAX + i];
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
      v += __shfl_down_sync(0xffffffffu, v, o);
   if ((threadIdx.x & 31) == 0)
      sh[threadIdx.x >> 5] = v;
   __syncthreads();
   for (int k = 0; k < ns; ++k)
      out[k] = sh[2 * k] + sh[2 * k + 1];
   __syncthreads();
}

// store this block's partial sum of v
static __device__ __forceinline__ void store_partial(double* red, int slot, double v, double* sh)
{
   v = block_sum(v, sh);
   if (threadIdx.x == 0)
      red[slot * RED_MAX + blockIdx.x] = v;
}

// store this block's partial sums of N values into slots first..first+N-1:
// the same shuffle trees as block_sum for each value (identical results), with
// the N values interleaved and one barrier pair instead of N (sh: >= 8 N
// doubles; blockDim <= 256)
template <int N>
static __device__ __forceinline__ void store_partials(double* red, int first, const double* v, double* sh)
{
   double x[N];
#pragma unroll
   for (int c = 0; c < N; ++c)
      x[c] = v[c];
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
#pragma unroll
      for (int c = 0; c < N; ++c)
         x[c] += __shfl_down_sync(0xffffffffu, x[c], o);
   const int w = threadIdx.x >> 5, l = threadIdx.x & 31, nw = blockDim.x >> 5;
   if (l == 0)
#pragma unroll
      for (int c = 0; c < N; ++c)
         sh[c * 8 + w] = x[c];
   __syncthreads();
   if (threadIdx.x < 32) {
#pragma unroll
      for (int c = 0; c < N; ++c) {
         double r = threadIdx.x < nw ? sh[c * 8 + threadIdx.x] : 0.0;
#pragma unroll
         for (int o = 16; o > 0; o >>= 1)
            r += __shfl_down_sync(0xffffffffu, r, o);
         if (threadIdx.x == 0)
            red[(first + c) * RED_MAX + blockIdx.x] = r;
      }
   }
   __syncthreads();
}

// true in the block that finishes last (threadfence + ticket); it resets the
// ticket for the next launch
static __device__ __forceinline__ bool last_block(int* ticket)
{
   __shared__ bool last;
   __threadfence();
   __syncthreads();
   if (threadIdx.x == 0) {
      unsigned prev = atomicAdd(reinterpret_cast<unsigned*>(ticket), 1u);
      last = prev == gridDim.x - 1;
   }
   __syncthreads();
   if (last) {
      __threadfence();
      if (threadIdx.x == 0)
         *ticket = 0;
   }
   return last;
}

}  // namespace t9gb
