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
// guess; ST_LREADY: bit 0 feature statistics, bit 1 target scale fixed,
// bit 3 statistics fixed in this solve (k_normalize writes the network input)
// ST_RANGE: a dipole-grid contribution reached the packed fixed-point guard;
// ST_RANGE_L: the same while evaluating the learned guess's residual;
// ST_TICKET_SUM: the last-block ticket of the energy / virial row sums;
// ST_LX: fits of the learned extrapolation so far (its coefficients replace
// the predictor's from the second on); ST_LX_REJ: fits whose solve failed
enum { ST_ITER = 0, ST_DONE, ST_STATUS, ST_NUALT, ST_TICKET0, ST_TICKET1, ST_LCHOICE, ST_LREADY, ST_RANGE,
   ST_RANGE_L, ST_TICKET_SUM, ST_LX, ST_LX_REJ, ST_NSTAT };
static_assert(ST_NSTAT <= 16, "the context allocates 16 status words");
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
   if (slot < ns) {
      // eight loads in flight per round; the additions keep the order of i
      const double* p = red + (first + slot) * RED_MAX;
      int i = sub;
      for (; i + 7 * 64 < nb; i += 8 * 64) {
         double t[8];
#pragma unroll
         for (int k = 0; k < 8; ++k)
            t[k] = p[i + k * 64];
#pragma unroll
         for (int k = 0; k < 8; ++k)
            v += t[k];
      }
      for (; i < nb; i += 64)
         v += p[i];
   }
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

// sum_slots for blocks of 128 or 256 threads: blockDim / 4 threads per slot
// (ns <= 4), the same fixed order for a given block size
static __device__ __forceinline__ void sum_slots_bd(const double* red, int first, int ns, int nb, double* sh,
   double* out)
{
   const int per = blockDim.x >> 2, wps = per >> 5;
   const int slot = threadIdx.x / per, sub = threadIdx.x % per;
   double v = 0;
   if (slot < ns) {
      const double* p = red + (first + slot) * RED_MAX;
      int i = sub;
      for (; i + 7 * per < nb; i += 8 * per) {
         double t[8];
#pragma unroll
         for (int k = 0; k < 8; ++k)
            t[k] = p[i + k * per];
#pragma unroll
         for (int k = 0; k < 8; ++k)
            v += t[k];
      }
      for (; i < nb; i += per)
         v += p[i];
   }
#pragma unroll
   for (int o = 16; o > 0; o >>= 1)
      v += __shfl_down_sync(0xffffffffu, v, o);
   if ((threadIdx.x & 31) == 0)
      sh[threadIdx.x >> 5] = v;
   __syncthreads();
   for (int k = 0; k < ns; ++k) {
      double t = 0;
      for (int w = 0; w < wps; ++w)
         t += sh[k * wps + w];
      out[k] = t;
   }
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

// store_partials for per-thread FP32 partials: the warp trees in FP32 (the
// FP64 pipe of this GPU issues a warp instruction in tens of cycles, so the
// per-thread and per-warp sums avoid it), the block's eight warp sums and
// everything after them in FP64; the same fixed order, so deterministic
template <int N>
static __device__ __forceinline__ void store_partials_f(double* red, int first, const float* v, double* sh)
{
   float x[N];
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
         sh[c * 8 + w] = (double)x[c];
   __syncthreads();
   if (threadIdx.x < N) {
      // one thread per value: the warp sums in order
      double r = 0.0;
      for (int k = 0; k < nw; ++k)
         r += sh[threadIdx.x * 8 + k];
      red[(first + threadIdx.x) * RED_MAX + blockIdx.x] = r;
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

// The CG scalars after the r.z / r.r sums (thread 0 of the last block).
// tot = {r.z d, r.z p, r.r d, r.r p}.  init: s = r.z, the first search
// direction is z itself (b = 0), counters reset.  Loop: b = s1 / s, s = s1,
// eps = debye sqrt(max(r.r) / n), iteration count, convergence (at least
// miniter, at most politer iterations), status, and the graph's WHILE
// condition (induceMutualPcg1_cu, src/cu/amoeba/pcg.cu:120-168).
__device__ __forceinline__ void pcg_scalars(const double* tot, double* scal, int* state, int init, int n,
   double debye, double poleps, int politer, int miniter, cudaGraphConditionalHandle handle, int use_handle)
{
   const double s1_d = tot[0], s1_p = tot[1], q_d = tot[2], q_p = tot[3];
   if (init) {
      scal[S_SUM_D] = s1_d;
      scal[S_SUM_P] = s1_p;
      scal[S_B_D] = 0.0;
      scal[S_B_P] = 0.0;
      state[ST_ITER] = 0;
      state[ST_DONE] = 0;
      state[ST_STATUS] = T9GB_OK;
      return;
   }
   // the ratios and the norm in FP32 from the FP64 sums: the kernels use
   // b as FP32, and an FP64 division or square root takes this GPU's FP64
   // pipe dozens of issue slots on the solve's critical path
   const double s_d = scal[S_SUM_D], s_p = scal[S_SUM_P];
   scal[S_B_D] = s_d == 0 ? 0.0 : (double)((float)s1_d / (float)s_d);
   scal[S_B_P] = s_p == 0 ? 0.0 : (double)((float)s1_p / (float)s_p);
   scal[S_SUM_D] = s1_d;
   scal[S_SUM_P] = s1_p;
   const double eps = (double)((float)debye * sqrtf((float)fmax(q_d, q_p) / (float)n));
   const int iter = state[ST_ITER] + 1;
   state[ST_ITER] = iter;
   bool done = eps < poleps;
   if (iter < miniter)
      done = false;
   if (iter >= politer)
      done = true;
   const bool nan = !(eps == eps);
   if (nan)
      done = true;
   scal[S_EPS] = eps;
   state[ST_DONE] = done ? 1 : 0;
   state[ST_STATUS] = nan ? T9GB_NAN_DETECTED : (done && !(eps < poleps) ? T9GB_NOT_CONVERGED : T9GB_OK);
   if (use_handle)
      cudaGraphSetConditional(handle, done ? 0u : 1u);
}

// Row s of the search direction p = z + b p_old formed where it is read
// (components 0-5: d with b_d, p with b_p; 6-7: the row's tags from p_old).
// Every reader forms it with the same fused multiply-add, so all see the
// same values.
__device__ __forceinline__ void dir_row(const float* __restrict__ p8, const float* __restrict__ z8, int s, float bd,
   float bp, float* v)
{
   const float4* p = reinterpret_cast<const float4*>(p8 + 8 * s);
   const float4* z = reinterpret_cast<const float4*>(z8 + 8 * s);
   const float4 p0 = p[0], p1 = p[1], z0 = z[0], z1 = z[1];
   v[0] = __fmaf_rn(bd, p0.x, z0.x);
   v[1] = __fmaf_rn(bd, p0.y, z0.y);
   v[2] = __fmaf_rn(bd, p0.z, z0.z);
   v[3] = __fmaf_rn(bp, p0.w, z0.w);
   v[4] = __fmaf_rn(bp, p1.x, z1.x);
   v[5] = __fmaf_rn(bp, p1.y, z1.y);
   v[6] = p1.z;
   v[7] = p1.w;
}

}  // namespace t9gb
