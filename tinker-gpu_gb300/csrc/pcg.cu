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
// calls and a host synchronisation (pcg.cu:144-145).  Here:
//  - dot products are FP64 block partials; the last block of the producing
//    kernel (threadfence + ticket) sums them in a fixed order and derives
//    the CG scalars, so results are bit-reproducible and no extra launch or
//    host round trip is needed;
//  - the convergence test, the iteration count and the predictor ring index
//    live on the device; the whole induce() -- neighbour list, permanent
//    field, guess, r0, the PCG loop as a conditional WHILE node, and the
//    predictor save -- is one CUDA graph, launched once per call.
#include <cmath>

#include "common.cuh"
#include "reduce.cuh"

namespace t9gb {

constexpr int VB = 256;  // vector-kernel block size

// ASPC extrapolation weights (Kolafa, J. Comput. Chem. 25, 335 (2004)); the
// reference tabulates them in src/cu/upredict.cu:40-55.
__constant__ double c_aspc[16] = {62. / 17., -310. / 51., 2170. / 323., -2329. / 400., 1701. / 409., -806. / 323.,
   1024. / 809., -479. / 883., 257. / 1316., -434. / 7429., 191. / 13375., -62. / 22287., 3. / 7217.,
   -3. / 67015., 2. / 646323., -1. / 9694845.};

// Gear 6-point extrapolation weights (the binomial coefficients of the
// fifth difference); the reference tabulates them in src/cu/upredict.cu:141-146.
__constant__ double c_gear[6] = {6., -15., 20., -15., 6., -1.};

struct VecArgs {
   int ne;   // 6 * npad active elements (d xyz, p xyz of each slot)
   int ne8;  // 8 * npad floats per vector (rows padded to 32 bytes)
   int nb;  // blocks of every vector kernel
   const float* polar;
   const float* polinv;
   int sparse;
};

// ---- start of induce ----

// E = field, udir = alpha E, guess: the predictor's extrapolation once its
// ring (depth 16 for ASPC, 6 for Gear) is full, else the direct guess
// alpha E (pcgguess) or zero
// coefficient of ring slot k (its frame's age j): ASPC / Gear, or the
// learned extrapolation's once it has two fits (lcoef: null when off)
__device__ __forceinline__ float ring_coef(int predictor, int j, const float* __restrict__ lcoef,
   const int* __restrict__ state)
{
   if (lcoef && state[ST_LX] >= 2)
      return lcoef[j];
   return (float)(predictor == 1 ? c_aspc[j] : c_gear[j]);
}

__global__ void k_init_guess(VecArgs A, const float* __restrict__ fld, float* __restrict__ efield,
   float* __restrict__ udir, float* __restrict__ uind, int pcgguess, int predictor, const float* __restrict__ hist,
   const int* __restrict__ state, int set_uind, const float* __restrict__ lcoef)
{
   const int nualt = state[ST_NUALT];
   const int depth = predictor == 1 ? 16 : predictor == 2 ? 6 : 0;
   const bool predict = depth > 0 && nualt >= depth;
   float coef[16];
   if (predict)
      for (int k = 0; k < depth; ++k) {
         const int j = ((nualt - 1 - k) % depth + depth) % depth;
         coef[k] = ring_coef(predictor, j, lcoef, state);
      }
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;  // row s, component e - 6 s of [npad][8]
      const float pol = A.polar[s];
      const float f = fld[x];
      efield[x] = f;
      const float ud = pol * f;
      udir[x] = ud;
      float u = 0.f;
      if (predict) {
         // FP32: the extrapolation's rounding is far below its own error
         float v = 0.f;
         for (int k = 0; k < depth; ++k)
            v = __fmaf_rn(coef[k], hist[(size_t)k * A.ne8 + x], v);
         u = v;
      } else if (pcgguess) {
         u = ud;
      }
      if (set_uind)
         uind[x] = u;
   }
}

// the predictor's guess alone (zero while its ring is not full), before the
// permanent field is known: the same extrapolation as k_init_guess
__global__ void k_predict(VecArgs A, int predictor, const float* __restrict__ hist, const int* __restrict__ state,
   float* __restrict__ uind, const float* __restrict__ lcoef)
{
   const int nualt = state[ST_NUALT];
   const int depth = predictor == 1 ? 16 : predictor == 2 ? 6 : 0;
   const bool predict = depth > 0 && nualt >= depth;
   float coef[16];
   if (predict)
      for (int k = 0; k < depth; ++k) {
         const int j = ((nualt - 1 - k) % depth + depth) % depth;
         coef[k] = ring_coef(predictor, j, lcoef, state);
      }
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;  // row s, component e - 6 s of [npad][8]
      float u = 0.f;
      if (predict) {
         // FP32: the extrapolation's rounding is far below its own error
         float v = 0.f;
         for (int k = 0; k < depth; ++k)
            v = __fmaf_rn(coef[k], hist[(size_t)k * A.ne8 + x], v);
         u = v;
      }
      uind[x] = u;
   }
}

// r0 = (udir - u0)/alpha + ufield(u0)  [= ufield(udir) for the direct guess,
// E for the zero guess]
__global__ void k_init_rsd(VecArgs A, const float* __restrict__ fld, const float* __restrict__ efield,
   const float* __restrict__ udir, const float* __restrict__ uind, float* __restrict__ rsd, int zero_guess)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;  // row s, component e - 6 s of [npad][8]
      float r = zero_guess ? efield[x] : (udir[x] - uind[x]) * A.polinv[s] + fld[x];
      if (A.polar[s] == 0.f)
         r = 0.f;
      rsd[x] = r;
   }
}

// z = M r (diagonal here, else read from the sparse kernel), p = z on init,
// partials r.z and r.r.  The last block: init -> s = r.z; loop -> b = s1/s,
// s = s1, eps, iteration count, convergence, graph condition.
__global__ void k_precond_dot(VecArgs A, const float* __restrict__ rsd, float* __restrict__ zrsd,
   float* __restrict__ conj, double* __restrict__ red, double* __restrict__ scal, int* __restrict__ state, int init,
   int n, double debye, double poleps, int politer, int miniter, cudaGraphConditionalHandle handle, int use_handle)
{
   __shared__ double sh[64];
   float rz_d = 0.f, rz_p = 0.f, rr_d = 0.f, rr_p = 0.f;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;  // row s, component e - 6 s of [npad][8]
      const float r = rsd[x];
      float z;
      if (A.sparse) {
         z = zrsd[x];
      } else {
         z = A.polar[s] * r;
         zrsd[x] = z;
      }
      if (init)
         conj[x] = z;
      if (e - 6 * s < 3) {
         rz_d += r * z;
         rr_d += r * r;
      } else {
         rz_p += r * z;
         rr_p += r * r;
      }
   }
   const float pv[4] = {rz_d, rz_p, rr_d, rr_p};
   store_partials_f<4>(red, R_RZ_D, pv, sh);
   if (!last_block(state + ST_TICKET0))
      return;
   double tot[4];
   sum_slots(red, R_RZ_D, 4, gridDim.x, sh, tot);
   if (threadIdx.x == 0)
      pcg_scalars(tot, scal, state, init, n, debye, poleps, politer, miniter, handle, use_handle);
}

// ---- loop body ----

// Ap = p/alpha - ufield(p); partials p.Ap; last block: a = s / p.Ap.
// DIR: p = z + b p_old is formed here (as the field kernels formed it) and
// stored.
// fld2 (may be null): the reciprocal + self part, stored apart from the
// real-space part in fld; the field is fld + fld2, the sum the gather forms
// when it adds itself to the real-space field.
template <bool DIR>
__global__ void k_pcg_p1(VecArgs A, const float* __restrict__ fld, const float* __restrict__ fld2,
   float* __restrict__ conj, const float* __restrict__ zrsd, float* __restrict__ vec, double* __restrict__ red,
   double* __restrict__ scal, int* __restrict__ state)
{
   pdl_wait();
   __shared__ double sh[64];
   float dd = 0.f, dp = 0.f;
   float bd = 0.f, bp = 0.f;
   if (DIR) {
      bd = (float)scal[S_B_D];
      bp = (float)scal[S_B_P];
   }
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;  // row s, component e - 6 s of [npad][8]
      float p = conj[x];
      if (DIR) {
         p = __fmaf_rn(e - 6 * s < 3 ? bd : bp, p, zrsd[x]);
         conj[x] = p;
      }
      const float f = fld2 ? fld[x] + fld2[x] : fld[x];
      const float v = A.polinv[s] * p - f;
      vec[x] = v;
      if (e - 6 * s < 3)
         dd += p * v;
      else
         dp += p * v;
   }
   const float pv[2] = {dd, dp};
   pdl_trigger();
   store_partials_f<2>(red, R_PAP_D, pv, sh);
   if (!last_block(state + ST_TICKET1))
      return;
   double tot[2];
   sum_slots(red, R_PAP_D, 2, gridDim.x, sh, tot);
   const double pap_d = tot[0], pap_p = tot[1];
   if (threadIdx.x == 0) {  // the step lengths in FP32 (used as FP32)
      scal[S_A_D] = pap_d == 0 ? 0.0 : (double)((float)scal[S_SUM_D] / (float)pap_d);
      scal[S_A_P] = pap_p == 0 ? 0.0 : (double)((float)scal[S_SUM_P] / (float)pap_p);
   }
}

// u += a p; r -= a Ap
__global__ void k_pcg_p2(VecArgs A, const double* __restrict__ scal, float* __restrict__ uind,
   const float* __restrict__ conj, float* __restrict__ rsd, const float* __restrict__ vec)
{
   pdl_wait();
   pdl_trigger();  // the preconditioner may stage its blocks
   const float a = (float)scal[S_A_D], ap = (float)scal[S_A_P];
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;  // row s, component e - 6 s of [npad][8]
      const float g = e - 6 * s < 3 ? a : ap;
      uind[x] += g * conj[x];
      float r = rsd[x] - g * vec[x];
      if (A.polar[s] == 0.f)
         r = 0.f;
      rsd[x] = r;
   }
}

// p = z + b p in place (the paths that do not form p where it is read)
__global__ void k_pcg_dir(VecArgs A, const double* __restrict__ scal, float* __restrict__ conj,
   const float* __restrict__ zrsd)
{
   pdl_wait();
   pdl_trigger();  // the spread may stage its blocks and form its B-splines
   const float b = (float)scal[S_B_D], bp = (float)scal[S_B_P];
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;  // row s, component e - 6 s of [npad][8]
      conj[x] = __fmaf_rn(e - 6 * s < 3 ? b : bp, conj[x], zrsd[x]);
   }
}

// after the loop: u += pcgpeek alpha r (induceMutualPcg1_cu,
// src/cu/amoeba/pcg.cu:170-178), and with a predictor the converged
// dipoles saved into its ring (ulspredSave, src/amoeba/induce.cpp:29-63)
__global__ void k_pcg_peek_save(VecArgs A, float* __restrict__ uind, const float* __restrict__ rsd, float pcgpeek,
   int depth, float* __restrict__ hist, const int* __restrict__ state)
{
   float* dst = depth > 0 ? hist + (size_t)(state[ST_NUALT] % depth) * A.ne8 : nullptr;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;  // row s, component e - 6 s of [npad][8]
      const float u = uind[x] + pcgpeek * A.polar[s] * rsd[x];
      uind[x] = u;
      if (dst)
         dst[x] = u;
   }
}

__global__ void k_bump_nualt(int* state, int depth)
{
   int v = state[ST_NUALT] + 1;
   if (v > 2 * depth)
      v -= depth;
   state[ST_NUALT] = v;
}

// ---------------------------------------------------------------------------

// Learned extrapolation of the predictor ring (t9gb_learn_extrapolation).
// After each solve the converged dipoles u_t (just saved in the ring) and
// the K frames before them give one least-squares sample per element of
// both dipole sets: u_t ~ sum_k a_k D^k u_{t-1}, D^k the k-th backward
// difference over the ring (a well-conditioned basis: Jacobi-scaled
// condition numbers of 10^2 - 10^3 at K = 6 - 8).  The normal equations are
// summed in a fixed order (FP32 per block, compensated FP32 across blocks),
// kept in FP64 with forgetting factor LX_LAMBDA, and solved by an FP32
// Cholesky in the launch's last block; the raw coefficients
// c_j = sum_k a_k (-1)^j C(k, j) of the ring frames replace the
// predictor's (ring_coef).  The PCG convergence test is unchanged.
constexpr int LX_MAXK = 8;
constexpr double LX_LAMBDA = 0.99;
constexpr int LX_NB = 152;                                // blocks of k_lx_train
constexpr int LX_NV = LX_MAXK * (LX_MAXK + 1) / 2 + LX_MAXK;  // partial sums per block

// signed binomials (-1)^j C(k, j), k, j < 8 (Pascal's triangle)
__constant__ float c_sbinom[LX_MAXK][LX_MAXK] = {
   {1, 0, 0, 0, 0, 0, 0, 0},
   {1, -1, 0, 0, 0, 0, 0, 0},
   {1, -2, 1, 0, 0, 0, 0, 0},
   {1, -3, 3, -1, 0, 0, 0, 0},
   {1, -4, 6, -4, 1, 0, 0, 0},
   {1, -5, 10, -10, 5, -1, 0, 0},
   {1, -6, 15, -20, 15, -6, 1, 0},
   {1, -7, 21, -35, 35, -21, 7, -1}};

// a + b = s + e exactly (Knuth's two-sum; the intrinsics keep the compiler
// from fusing or reordering the sums): returns e and writes s to out, which
// may alias a
__device__ __forceinline__ float two_sum(float a, float b, float& out)
{
   const float s = __fadd_rn(a, b);
   const float bb = __fsub_rn(s, a);
   const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
   out = s;
   return e;
}

// Cholesky solve of the Jacobi-scaled normal equations (M + ridge I) z = r
// in FP32 (M = S A S, r = S b, S = diag(sc)); false when a pivot is not
// positive.  r returns the unscaled solution S z.
template <int K>
__device__ bool lx_solve(const float (*Ms)[K + 1], const float* sc, float ridge, float* r)
{
   float M[K][K];
#pragma unroll
   for (int k = 0; k < K; ++k) {
#pragma unroll
      for (int q = 0; q < K; ++q)
         M[k][q] = Ms[k][q] * sc[k] * sc[q] + (k == q ? ridge : 0.f);
      r[k] = Ms[k][K] * sc[k];
   }
   // M = L L^T in place (lower), then L z = r, L^T a = z
#pragma unroll
   for (int k = 0; k < K; ++k) {
      float dkk = M[k][k];
#pragma unroll
      for (int q = 0; q < k; ++q)
         dkk -= M[k][q] * M[k][q];
      if (!(dkk > 0.f))
         return false;
      dkk = sqrtf(dkk);
      M[k][k] = dkk;
      const float inv = 1.f / dkk;
#pragma unroll
      for (int i = k + 1; i < K; ++i) {
         float t = M[i][k];
#pragma unroll
         for (int q = 0; q < k; ++q)
            t -= M[i][q] * M[k][q];
         M[i][k] = t * inv;
      }
   }
#pragma unroll
   for (int k = 0; k < K; ++k) {
      float t = r[k];
#pragma unroll
      for (int q = 0; q < k; ++q)
         t -= M[k][q] * r[q];
      r[k] = t / M[k][k];
   }
#pragma unroll
   for (int k = K - 1; k >= 0; --k) {
      float t = r[k];
#pragma unroll
      for (int q = k + 1; q < K; ++q)
         t -= M[q][k] * r[q];
      r[k] = t / M[k][k];
   }
#pragma unroll
   for (int k = 0; k < K; ++k)
      r[k] *= sc[k];
   return true;
}

// The differences are formed in FP32 (each subtraction rounds to its own
// result) and the products summed in FP32 per thread and block (a few
// hundred terms).  FP64 runs at 1/64 of the FP32 rate on this GPU: FP64
// differences and FP64 cross-block sums made the kernel 20.8 us at 12,288
// atoms, against 10.7 us now.
template <int K>
__global__ void __launch_bounds__(256) k_lx_train(VecArgs A, const float* __restrict__ hist, float* __restrict__ part,
   double* __restrict__ lx, float* __restrict__ lcoef, int* __restrict__ state, int* __restrict__ ticket, int depth)
{
   constexpr int NV = K * (K + 1) / 2 + K;
   __shared__ float sh[8][NV];
   const int nualt = state[ST_NUALT] - 1;  // after the solve's bump: the new frame is slot nualt % depth
   if (nualt < K)
      return;  // every block alike
   float acc[NV];
#pragma unroll
   for (int v = 0; v < NV; ++v)
      acc[v] = 0.f;
   const float* fy = hist + (size_t)(nualt % depth) * A.ne8;
   const float* fr[K];
#pragma unroll
   for (int j = 0; j < K; ++j)
      fr[j] = hist + (size_t)(((nualt - 1 - j) % depth + depth) % depth) * A.ne8;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < A.ne; e += gridDim.x * blockDim.x) {
      const int s = e / 6, x = e + 2 * s;
      float t[K];
#pragma unroll
      for (int j = 0; j < K; ++j)
         t[j] = fr[j][x];
      float d[K];
#pragma unroll
      for (int k = 0; k < K; ++k) {  // the difference table: d_k = sum_j (-1)^j C(k, j) u_j
         d[k] = t[0];
#pragma unroll
         for (int j = 0; j + 1 < K - k; ++j)
            t[j] -= t[j + 1];
      }
      const float y = fy[x];
      int v = 0;
#pragma unroll
      for (int k = 0; k < K; ++k) {
#pragma unroll
         for (int l = 0; l <= k; ++l)
            acc[v++] += d[k] * d[l];
      }
#pragma unroll
      for (int k = 0; k < K; ++k)
         acc[v++] += d[k] * y;
   }
   // block sums (warp trees, then the eight warps in order), one row per block
   const int w = threadIdx.x >> 5, l = threadIdx.x & 31;
#pragma unroll
   for (int v = 0; v < NV; ++v) {
      float a = acc[v];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         a += __shfl_xor_sync(0xffffffffu, a, o);
      if (l == 0)
         sh[w][v] = a;
   }
   __syncthreads();
   for (int v = threadIdx.x; v < NV; v += blockDim.x)
      part[(size_t)v * LX_NB + blockIdx.x] =
         ((sh[0][v] + sh[1][v]) + (sh[2][v] + sh[3][v])) + ((sh[4][v] + sh[5][v]) + (sh[6][v] + sh[7][v]));
   if (!last_block(ticket))
      return;
   // the block partials: warp w sums values w, w + 8, ..., every lane over
   // the blocks lane + 32 i in order, then a fixed butterfly, in compensated
   // FP32 (the sum and its exact rounding errors, two_sum): as accurate as
   // FP64 here, which runs at 1/64 of the FP32 rate on this GPU
   constexpr int NVW = (NV + 7) / 8, NBL = (LX_NB + 31) / 32;
   __shared__ float tot_s[NV], tot_c[NV];
   float pv[NVW][NBL];
#pragma unroll
   for (int i = 0; i < NVW; ++i)
#pragma unroll
      for (int q = 0; q < NBL; ++q) {
         const int v = w + 8 * i, b = l + 32 * q;
         pv[i][q] = v < NV && b < LX_NB ? __ldcg(part + (size_t)v * LX_NB + b) : 0.f;
      }
#pragma unroll
   for (int i = 0; i < NVW; ++i) {
      float a = pv[i][0], c = 0.f;
#pragma unroll
      for (int q = 1; q < NBL; ++q)
         c += two_sum(a, pv[i][q], a);
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
         const float a2 = __shfl_xor_sync(0xffffffffu, a, o), c2 = __shfl_xor_sync(0xffffffffu, c, o);
         const float e = two_sum(a, a2, a);
         c = (c + c2) + e;
      }
      if (l == 0 && w + 8 * i < NV) {
         tot_s[w + 8 * i] = a;
         tot_c[w + 8 * i] = c;
      }
   }
   __syncthreads();
   // normal equations with forgetting (FP64), one entry per thread:
   // lx = [A, b]; the system in FP32 into shared memory for the solve
   __shared__ float Ms[K][K + 1];
   for (int v = threadIdx.x; v < NV; v += blockDim.x) {
      int k, q;
      if (v < K * (K + 1) / 2) {
         k = 0;
         while ((k + 1) * (k + 2) / 2 <= v)
            ++k;
         q = v - k * (k + 1) / 2;
      } else {
         k = v - K * (K + 1) / 2;
         q = K;
      }
      const int at = q < K ? k * LX_MAXK + q : LX_MAXK * LX_MAXK + k;
      const double a = LX_LAMBDA * lx[at] + ((double)tot_s[v] + (double)tot_c[v]);
      lx[at] = a;
      const float af = (float)a;
      if (q < K) {
         lx[q * LX_MAXK + k] = a;
         Ms[k][q] = af;
         Ms[q][k] = af;
      } else {
         Ms[k][K] = af;
      }
   }
   __syncthreads();
   if (threadIdx.x != 0)
      return;
   // the Jacobi-scaled system (condition numbers 10 - 10^3) in FP32: the
   // sums above carry FP64 accuracy, the solve needs no more.  A failed
   // factorisation retries with a 100x larger ridge (twice), then leaves the
   // previous coefficients in place and counts the rejection.
   float sc[K], r[K];
   bool ok = true;
   for (int k = 0; k < K; ++k) {
      const float a = Ms[k][k];
      ok = ok && a > 0.f;  // no information yet: the predictor's coefficients stay
      sc[k] = ok ? rsqrtf(a) : 0.f;
   }
   if (ok) {
      ok = false;
      for (float ridge = 1e-6f; !ok && ridge < 1e-1f; ridge *= 100.f)
         ok = lx_solve<K>(Ms, sc, ridge, r);
   }
   if (!ok) {
      state[ST_LX_REJ] = min(state[ST_LX_REJ] + 1, 1 << 20);
      return;
   }
   float cf[16];
   for (int j = 0; j < 16; ++j) {
      float c = 0.f;
      if (j < K)
         for (int k = j; k < K; ++k)
            c += r[k] * c_sbinom[k][j];
      cf[j] = c;
   }
   for (int j = 0; j < 16; ++j)
      lcoef[j] = cf[j];
   state[ST_LX] = min(state[ST_LX] + 1, 1 << 20);
}

static VecArgs vec_args(const Context* ctx)
{
   VecArgs A;
   A.ne = 6 * ctx->npad;
   A.ne8 = 8 * ctx->npad;
   A.nb = std::min(RED_MAX, grid_for(A.ne, VB));
   A.polar = ctx->spolar;
   A.polinv = ctx->spolinv;
   A.sparse = ctx->cfg.pcgprec ? 1 : 0;
   return A;
}

// ---------------------------------------------------------------------------
// Verlet reuse of the neighbour list.  The list holds the pairs within
// cutoff + buffer at its build; it stays valid while every atom is within
// half the buffer of its position at the build.  It is rebuilt when the host
// requests it (new order, grown capacity, overflow) or when the device check
// finds an atom that moved further.  Inside the induce() graph the decision
// is a conditional IF node set by the check kernel; the host-driven path
// reads the same flag, so both paths make the same decisions.

__global__ void k_disp_check(int npad, const float4* __restrict__ spos, const float4* __restrict__ sref, float lx,
   float ly, float lz, float ilx, float ily, float ilz, float lim2, int* __restrict__ flag, int* __restrict__ state,
   cudaGraphConditionalHandle handle, int use_handle)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      const float4 a = spos[s], b = sref[s];
      const float dx = image1(a.x - b.x, lx, ilx), dy = image1(a.y - b.y, ly, ily), dz = image1(a.z - b.z, lz, ilz);
      if (dx * dx + dy * dy + dz * dz > lim2)
         atomicOr(flag, 1);
   }
   if (!last_block(state + ST_TICKET0))
      return;
   if (threadIdx.x == 0 && use_handle)
      cudaGraphSetConditional(handle, *(volatile int*)flag ? 1u : 0u);
}

__global__ void k_list_done(int npad, const float4* __restrict__ spos, float4* __restrict__ sref, int* __restrict__ flag)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x)
      sref[s] = spos[s];
   if (blockIdx.x == 0 && threadIdx.x == 0)
      *flag = 0;
}

static int list_request(Context* ctx)
{
   if (ctx->list_need_build) {
      T9_CUDA(cudaMemsetAsync(ctx->lflag, 0xff, sizeof(int), ctx->stream));
      ctx->list_need_build = false;
   }
   return T9GB_OK;
}

static int launch_disp_check(Context* ctx, cudaGraphConditionalHandle handle, int use_handle)
{
   const t9gb_config& c = ctx->cfg;
   const bool pbc = c.box[0] > 0 && c.box[1] > 0 && c.box[2] > 0;
   const float half = 0.5f * (float)c.list_buffer;
   const int nb = std::min(RED_MAX, grid_for(ctx->npad, 256));
   k_disp_check<<<nb, 256, 0, ctx->stream>>>(ctx->npad, ctx->spos, ctx->sref, pbc ? (float)c.box[0] : 0.f,
      pbc ? (float)c.box[1] : 0.f, pbc ? (float)c.box[2] : 0.f, pbc ? (float)(1.0 / c.box[0]) : 0.f,
      pbc ? (float)(1.0 / c.box[1]) : 0.f, pbc ? (float)(1.0 / c.box[2]) : 0.f, half * half, ctx->lflag, ctx->status,
      handle, use_handle);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

static int list_build_body(Context* ctx)
{
   T9_CHECK(list_update(ctx));
   k_list_done<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, ctx->spos, ctx->sref, ctx->lflag);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// host-driven refresh (one synchronisation)
int ensure_list(Context* ctx)
{
   if (!ctx->list_stale && !ctx->list_need_build)
      return T9GB_OK;
   T9_CHECK(list_request(ctx));
   T9_CHECK(launch_disp_check(ctx, 0, 0));
   T9_CUDA(cudaMemcpyAsync(ctx->h_lflag, ctx->lflag, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   if (*ctx->h_lflag)
      T9_CHECK(list_build_body(ctx));
   T9_CHECK(launch_list_filter(ctx));
   T9_CUDA(cudaMemcpyAsync(ctx->h_over, ctx->nbr_over, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
   ctx->list_stale = false;
   return T9GB_OK;
}

// the same inside a stream capture: check kernel, then a conditional IF node
// whose body rebuilds the list
static int list_refresh_graph(Context* ctx)
{
   cudaStream_t s0 = ctx->stream;
   cudaStreamCaptureStatus cs;
   cudaGraph_t cap = nullptr;
   const cudaGraphNode_t* deps = nullptr;
   size_t ndeps = 0;
   if (cudaStreamGetCaptureInfo(s0, &cs, nullptr, &cap, &deps, nullptr, &ndeps) != cudaSuccess)
      return T9GB_CUDA_ERR;
   cudaGraphConditionalHandle handle = 0;
   T9_CUDA(cudaGraphConditionalHandleCreate(&handle, cap, 0, cudaGraphCondAssignDefault));
   T9_CHECK(launch_disp_check(ctx, handle, 1));
   if (cudaStreamGetCaptureInfo(s0, &cs, nullptr, &cap, &deps, nullptr, &ndeps) != cudaSuccess)
      return T9GB_CUDA_ERR;
   cudaGraphNodeParams cp = {};
   cp.type = cudaGraphNodeTypeConditional;
   cp.conditional.handle = handle;
   cp.conditional.type = cudaGraphCondTypeIf;
   cp.conditional.size = 1;
   cudaGraphNode_t node = nullptr;
   T9_CUDA(cudaGraphAddNode(&node, cap, deps, nullptr, ndeps, &cp));
   T9_CUDA(cudaStreamUpdateCaptureDependencies(s0, &node, nullptr, 1, cudaStreamSetCaptureDependencies));
   if (!ctx->cap_stream)
      T9_CUDA(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
   cudaGraph_t body = cp.conditional.phGraph_out[0];
   T9_CUDA(cudaStreamBeginCaptureToGraph(ctx->cap_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal));
   ctx->stream = ctx->cap_stream;
   int rc = list_build_body(ctx);
   ctx->stream = s0;
   cudaGraph_t tmp = nullptr;
   if (cudaStreamEndCapture(ctx->cap_stream, &tmp) != cudaSuccess && rc == T9GB_OK)
      rc = T9GB_CUDA_ERR;
   T9_CHECK(rc);
   T9_CHECK(launch_list_filter(ctx));
   T9_CUDA(cudaMemcpyAsync(ctx->h_over, ctx->nbr_over, sizeof(int), cudaMemcpyDeviceToHost, s0));
   return T9GB_OK;
}

// after a synchronisation: grow the list if an atom had more neighbours than
// the row capacity; *redo = 1 when the caller must repeat its work
int check_list_overflow(Context* ctx, int* redo)
{
   *redo = 0;
   if (*ctx->h_over <= ctx->nbr_cap)
      return T9GB_OK;
   int cap = ((int)(*ctx->h_over * 1.25) + 31) / 32 * 32;
   T9_CHECK(alloc_lists(ctx, cap));
   *ctx->h_over = 0;
   T9_CUDA(cudaMemsetAsync(ctx->nbr_over, 0, sizeof(int), ctx->stream));
   ctx->list_need_build = true;
   drop_graphs(ctx);
   *redo = 1;
   return T9GB_OK;
}

// The reciprocal grid (spread + transform) runs on the side stream while the
// real-space pair kernel runs on ctx->stream; after the join the gather adds
// recip + self to the real-space field (the same sum, so the same bits, as
// the serial order).  Serial while the per-kernel profile is on.
int side_index(const Context* ctx)
{
   return ctx->cap_stream && ctx->stream == ctx->cap_stream ? 1 : 0;
}

int recip_fork(Context* ctx, int k)
{
   T9_CUDA(cudaEventRecord(ctx->ev_fork[k], ctx->stream));
   T9_CUDA(cudaStreamWaitEvent(ctx->side_stream[k], ctx->ev_fork[k], 0));
   return T9GB_OK;
}

int recip_join(Context* ctx, int k)
{
   T9_CUDA(cudaEventRecord(ctx->ev_join[k], ctx->side_stream[k]));
   T9_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_join[k], 0));
   return T9GB_OK;
}

static int ufield6(Context* ctx, const float* u6, float* out6)
{
   if (!ctx->cfg.use_ewald)
      return launch_ufield_real(ctx, u6, nullptr, out6);
   if (ctx->prof.on) {
      T9_CHECK(launch_ufield_recip(ctx, u6, ctx->rcp6));
      return launch_ufield_real(ctx, u6, ctx->rcp6, out6);
   }
   const int k = side_index(ctx);
   T9_CHECK(recip_fork(ctx, k));
   cudaStream_t main = ctx->stream;
   ctx->stream = ctx->side_stream[k];
   const int rc = launch_ufield_recip_grid(ctx, u6);
   ctx->stream = main;
   T9_CHECK(rc);
   T9_CHECK(launch_ufield_real(ctx, u6, nullptr, out6));
   T9_CHECK(recip_join(ctx, k));
   return launch_ufield_recip_gather(ctx, u6, out6, true);
}

static int dfield6(Context* ctx, float* out6)
{
   if (!ctx->cfg.use_ewald)
      return launch_dfield_real(ctx, nullptr, out6);
   if (ctx->prof.on) {
      T9_CHECK(launch_dfield_recip(ctx, ctx->rcp6));
      return launch_dfield_real(ctx, ctx->rcp6, out6);
   }
   const int k = side_index(ctx);
   T9_CHECK(recip_fork(ctx, k));
   cudaStream_t main = ctx->stream;
   ctx->stream = ctx->side_stream[k];
   const int rc = launch_dfield_recip_grid(ctx);
   ctx->stream = main;
   T9_CHECK(rc);
   T9_CHECK(launch_dfield_real(ctx, nullptr, out6));
   T9_CHECK(recip_join(ctx, k));
   return launch_dfield_recip_gather(ctx, out6, true);
}

// z = M r with r.z, r.r and the CG scalars: one fused kernel for the sparse
// preconditioner, else the preconditioner and the dot kernel
static int precond_dots(Context* ctx, const VecArgs& A, int init, cudaGraphConditionalHandle handle,
   int use_handle)
{
   const t9gb_config& c = ctx->cfg;
   const int miniter = init ? 3 : std::min(3, ctx->n);
   if (A.sparse && (ctx->pcg_fuse & 1)) {
      PcgDots D{ctx->conj, ctx->red, ctx->scal, ctx->status, init, ctx->n, c.debye, c.poleps, c.politer, miniter,
         handle, use_handle};
      return launch_precond_sparse_dots(ctx, ctx->rsd, ctx->zrsd, D);
   }
   if (A.sparse)
      T9_CHECK(launch_precond_sparse(ctx, ctx->rsd, ctx->zrsd));
   prof_begin(ctx, P_VECTOR);
   k_precond_dot<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->rsd, ctx->zrsd, ctx->conj, ctx->red, ctx->scal, ctx->status,
      init, ctx->n, c.debye, c.poleps, c.politer, miniter, handle, use_handle);
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// One CG iteration.  With PME outside profiling the search direction
// p = z + b p_old is formed by its readers (spread, real-space field,
// gather) and the gather also forms Ap = p/alpha - ufield(p), p.Ap and a,
// storing p; elsewhere p is formed first and Ap by its own kernel.  Then
// u += a p, r -= a Ap, and the preconditioner with the dots.
static int pcg_body(Context* ctx, const VecArgs& A, cudaGraphConditionalHandle handle, int use_handle)
{
   if (ctx->cfg.use_ewald && (ctx->pcg_fuse & 2) && !ctx->prof.on) {
      const int k = side_index(ctx);
      T9_CHECK(recip_fork(ctx, k));
      cudaStream_t main = ctx->stream;
      ctx->stream = ctx->side_stream[k];
      const int rc = launch_ufield_recip_grid_dir(ctx, ctx->conj, ctx->zrsd, ctx->scal);
      ctx->stream = main;
      T9_CHECK(rc);
      T9_CHECK(launch_ufield_real_dir(ctx, ctx->conj, ctx->zrsd, ctx->scal, ctx->fld6));
      T9_CHECK(recip_join(ctx, k));
      PcgAp P{ctx->zrsd, ctx->conj, A.polinv, ctx->vec, ctx->red, ctx->scal, ctx->status};
      if (ctx->pcg_fuse & 4) {
         T9_CHECK(launch_ufield_recip_gather_ap(ctx, ctx->fld6, P));
      } else {
         T9_CHECK(launch_ufield_recip_gather_dir(ctx, ctx->fld6, P));
         k_pcg_p1<true><<<A.nb, VB, 0, ctx->stream>>>(A, ctx->fld6, nullptr, ctx->conj, ctx->zrsd, ctx->vec,
            ctx->red, ctx->scal, ctx->status);
      }
   } else {
      const bool pdl = use_pdl(ctx);
      prof_begin(ctx, P_VECTOR);
      T9_CUDA(launch_k(pdl, k_pcg_dir, A.nb, VB, 0, ctx->stream, A, ctx->scal, ctx->conj, ctx->zrsd));
      prof_end(ctx);
      const float* rcp = nullptr;
      if (ctx->cfg.use_ewald && (ctx->pcg_fuse & 96) == 96 && !ctx->prof.on) {
         // the reciprocal chain (spread, transform passes, gather into rcp6)
         // stays on this stream as programmatic dependents of the direction
         // kernel; the real-space field runs on the side stream
         const int k = side_index(ctx);
         T9_CHECK(recip_fork(ctx, k));
         cudaStream_t main = ctx->stream;
         ctx->stream = ctx->side_stream[k];
         int rc = launch_ufield_real(ctx, ctx->conj, nullptr, ctx->fld6);
         ctx->stream = main;
         T9_CHECK(rc);
         T9_CHECK(launch_ufield_recip_grid(ctx, ctx->conj));
         T9_CHECK(launch_ufield_recip_gather(ctx, ctx->conj, ctx->rcp6, false));
         T9_CHECK(recip_join(ctx, k));
         rcp = ctx->rcp6;
      } else if (ctx->cfg.use_ewald && (ctx->pcg_fuse & 32) && !ctx->prof.on) {
         // the gather follows the transform on the side stream (a programmatic
         // dependent of its last pass, so its position-only prologue overlaps
         // it) into rcp6; the Ap kernel adds it to the real-space field
         const int k = side_index(ctx);
         T9_CHECK(recip_fork(ctx, k));
         cudaStream_t main = ctx->stream;
         ctx->stream = ctx->side_stream[k];
         int rc = launch_ufield_recip_grid(ctx, ctx->conj);
         if (rc == T9GB_OK)
            rc = launch_ufield_recip_gather(ctx, ctx->conj, ctx->rcp6, false);
         ctx->stream = main;
         T9_CHECK(rc);
         T9_CHECK(launch_ufield_real(ctx, ctx->conj, nullptr, ctx->fld6));
         T9_CHECK(recip_join(ctx, k));
         rcp = ctx->rcp6;
      } else {
         T9_CHECK(ufield6(ctx, ctx->conj, ctx->fld6));
      }
      prof_begin(ctx, P_VECTOR);
      T9_CUDA(launch_k(pdl, k_pcg_p1<false>, A.nb, VB, 0, ctx->stream, A, ctx->fld6, rcp, ctx->conj, nullptr,
         ctx->vec, ctx->red, ctx->scal, ctx->status));
      prof_end(ctx);
   }
   prof_begin(ctx, P_VECTOR);
   T9_CUDA(launch_k(use_pdl(ctx), k_pcg_p2, A.nb, VB, 0, ctx->stream, A, ctx->scal, ctx->uind, ctx->conj, ctx->rsd,
      ctx->vec));
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return precond_dots(ctx, A, 0, handle, use_handle);
}

// start variants: the plain guess (ASPC / alpha E / zero), the learned guess
// for both systems, or both with the per-system residual comparison
// V_PREDICT: the plain start with the predictor's ring full, the field of
// the extrapolated guess computed beside the permanent field
enum { V_PLAIN = 0, V_LEARNED = 1, V_COMPARE = 2, V_PREDICT = 3 };

// V_PREDICT: the guess does not depend on this step's permanent field, so
// its mutual field (real space on side stream 2, the reciprocal grid on side
// stream 3 and the second grid, the gather back on stream 2) runs beside the
// permanent field (main and side stream 0), and both reciprocal grids beside
// the neighbour-list refresh; the same kernels and sums as the plain start,
// so the same bits
static int pcg_start_predict(Context* ctx, const VecArgs& A, bool graph)
{
   const t9gb_config& c = ctx->cfg;
   k_predict<<<A.nb, VB, 0, ctx->stream>>>(A, c.predictor, ctx->aspc_hist, ctx->status, ctx->uind, ctx->lx_coef);
   T9_CUDA(cudaGetLastError());
   // the two reciprocal grids need no neighbour list: they start first and
   // run beside the list refresh (side 0: the permanent grid; side 3: the
   // guess's grid on the second grid pair)
   T9_CHECK(recip_fork(ctx, 0));
   T9_CHECK(recip_fork(ctx, 3));
   cudaStream_t main = ctx->stream;
   ctx->stream = ctx->side_stream[0];
   int rc = launch_dfield_recip_grid(ctx);
   if (rc == T9GB_OK) {
      ctx->stream = ctx->side_stream[3];
      rc = launch_ufield_recip_grid_alt(ctx, ctx->uind);
   }
   ctx->stream = main;
   T9_CHECK(rc);
   T9_CHECK(graph ? list_refresh_graph(ctx) : ensure_list(ctx));
   // the real-space fields: the guess's on side 2 (then its gather, after the
   // grid), the permanent one here (then its gather)
   T9_CHECK(recip_fork(ctx, 2));
   ctx->stream = ctx->side_stream[2];
   rc = launch_ufield_real(ctx, ctx->uind, nullptr, ctx->tmp6);
   if (rc == T9GB_OK && cudaEventRecord(ctx->ev_join[3], ctx->side_stream[3]) == cudaSuccess &&
      cudaStreamWaitEvent(ctx->side_stream[2], ctx->ev_join[3], 0) == cudaSuccess)
      rc = launch_ufield_recip_gather_alt(ctx, ctx->uind, ctx->tmp6);
   else if (rc == T9GB_OK)
      rc = T9GB_CUDA_ERR;
   ctx->stream = main;
   T9_CHECK(rc);
   T9_CHECK(launch_dfield_real(ctx, nullptr, ctx->fld6));
   T9_CHECK(recip_join(ctx, 0));
   T9_CHECK(launch_dfield_recip_gather(ctx, ctx->fld6, true));
   T9_CHECK(recip_join(ctx, 2));
   k_init_guess<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->fld6, ctx->efield, ctx->udir, ctx->uind, c.pcgguess,
      c.predictor, ctx->aspc_hist, ctx->status, 0, ctx->lx_coef);
   if (ctx->learn_mode & 1)
      T9_CHECK(learn_forward(ctx, false));
   k_init_rsd<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->tmp6, ctx->efield, ctx->udir, ctx->uind, ctx->rsd, 0);
   T9_CUDA(cudaGetLastError());
   return precond_dots(ctx, A, 1, 0, 0);
}

// neighbour list, permanent field, guess, r0, M r0 and s = r.z
static int pcg_start(Context* ctx, const VecArgs& A, bool graph, int variant)
{
   const t9gb_config& c = ctx->cfg;
   if (variant == V_PREDICT)
      return pcg_start_predict(ctx, A, graph);
   if (c.use_ewald && !ctx->prof.on) {
      // the permanent grid needs no neighbour list: it runs beside the refresh
      T9_CHECK(recip_fork(ctx, 0));
      cudaStream_t main = ctx->stream;
      ctx->stream = ctx->side_stream[0];
      const int rc = launch_dfield_recip_grid(ctx);
      ctx->stream = main;
      T9_CHECK(rc);
      T9_CHECK(graph ? list_refresh_graph(ctx) : ensure_list(ctx));
      T9_CHECK(launch_dfield_real(ctx, nullptr, ctx->fld6));
      T9_CHECK(recip_join(ctx, 0));
      T9_CHECK(launch_dfield_recip_gather(ctx, ctx->fld6, true));
   } else {
      T9_CHECK(graph ? list_refresh_graph(ctx) : ensure_list(ctx));
      T9_CHECK(dfield6(ctx, ctx->fld6));
   }
   k_init_guess<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->fld6, ctx->efield, ctx->udir, ctx->uind, c.pcgguess,
      c.predictor, ctx->aspc_hist, ctx->status, 1, ctx->lx_coef);
   // the network runs when its guess is used or when this solve trains it
   if ((ctx->learn_mode & 1) || variant != V_PLAIN)
      T9_CHECK(learn_forward(ctx, variant != V_PLAIN));
   if (variant == V_LEARNED)
      T9_CHECK(learn_guess(ctx, ctx->uind, 1));
   else if (variant == V_COMPARE)
      T9_CHECK(learn_guess(ctx, ctx->tmp6, 0));
   const bool zero_guess = !c.pcgguess && pred_depth(c) == 0 && variant != V_LEARNED;
   if (!zero_guess)
      T9_CHECK(ufield6(ctx, ctx->uind, ctx->fld6));
   k_init_rsd<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->fld6, ctx->efield, ctx->udir, ctx->uind, ctx->rsd,
      zero_guess ? 1 : 0);
   if (variant == V_COMPARE) {
      // residual of the learned guess; each of d, p starts from the smaller
      // (a learned guess beyond the grid's fixed-point range is rejected)
      ctx->pme.probe = true;
      const int rc = ufield6(ctx, ctx->tmp6, ctx->vec);
      ctx->pme.probe = false;
      T9_CHECK(rc);
      T9_CHECK(learn_pick(ctx, ctx->tmp6, ctx->vec));
   }
   return precond_dots(ctx, A, 1, 0, 0);
}

static int pcg_finish(Context* ctx, const VecArgs& A)
{
   const int depth = pred_depth(ctx->cfg);
   if (ctx->cfg.pcgpeek != 0.0 || depth > 0) {
      k_pcg_peek_save<<<A.nb, VB, 0, ctx->stream>>>(A, ctx->uind, ctx->rsd, (float)ctx->cfg.pcgpeek, depth,
         ctx->aspc_hist, ctx->status);
      T9_CUDA(cudaGetLastError());
   }
   if (depth > 0)
      k_bump_nualt<<<1, 1, 0, ctx->stream>>>(ctx->status, depth);
   if (ctx->learn_mode & 1)
      T9_CHECK(learn_train(ctx));
   T9_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->status, sizeof(int) * ST_NSTAT, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaMemcpyAsync(ctx->h_scal, ctx->scal, sizeof(double) * S_NSCAL, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// host-driven loop (used while profiling: every launch is bracketed)
static int induce_stepwise(Context* ctx, int variant)
{
   const VecArgs A = vec_args(ctx);
   T9_CHECK(pcg_start(ctx, A, false, variant));
   const int politer = std::max(1, ctx->cfg.politer);
   for (int it = 0; it < politer; ++it) {
      T9_CHECK(pcg_body(ctx, A, 0, 0));
      T9_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->status, sizeof(int) * ST_NSTAT, cudaMemcpyDeviceToHost,
         ctx->stream));
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
      if (ctx->h_status[ST_DONE])
         break;
   }
   T9_CHECK(pcg_finish(ctx, A));
   if (ctx->stage_out)
      T9_CHECK(stage_dipoles(ctx));
   else if (ctx->out_d || ctx->out_p)
      T9_CHECK(scatter_from_sorted3(ctx, ctx->uind, ctx->out_d, ctx->out_p));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return T9GB_OK;
}

// capture the whole induce() into one graph with a conditional WHILE loop
static int induce_capture(Context* ctx, int variant)
{
   const VecArgs A = vec_args(ctx);
   cudaStream_t s0 = ctx->stream;
   if (!ctx->cap_stream)
      T9_CUDA(cudaStreamCreateWithFlags(&ctx->cap_stream, cudaStreamNonBlocking));
   cudaGraph_t graph = nullptr;
   T9_CUDA(cudaStreamBeginCapture(s0, cudaStreamCaptureModeThreadLocal));
   int rc = pcg_start(ctx, A, true, variant);
   cudaStreamCaptureStatus cs;
   cudaGraph_t cap = nullptr;
   const cudaGraphNode_t* deps = nullptr;
   size_t ndeps = 0;
   cudaGraphConditionalHandle handle = 0;
   cudaGraphNode_t cnode = nullptr;
   cudaGraphNodeParams cp = {};
   if (rc == T9GB_OK && cudaStreamGetCaptureInfo(s0, &cs, nullptr, &cap, &deps, nullptr, &ndeps) != cudaSuccess)
      rc = T9GB_CUDA_ERR;
   if (rc == T9GB_OK && cudaGraphConditionalHandleCreate(&handle, cap, 1, cudaGraphCondAssignDefault) != cudaSuccess)
      rc = T9GB_CUDA_ERR;
   if (rc == T9GB_OK) {
      cp.type = cudaGraphNodeTypeConditional;
      cp.conditional.handle = handle;
      cp.conditional.type = cudaGraphCondTypeWhile;
      cp.conditional.size = 1;
      if (cudaGraphAddNode(&cnode, cap, deps, nullptr, ndeps, &cp) != cudaSuccess)
         rc = T9GB_CUDA_ERR;
   }
   if (rc == T9GB_OK && cudaStreamUpdateCaptureDependencies(s0, &cnode, nullptr, 1, cudaStreamSetCaptureDependencies)
         != cudaSuccess)
      rc = T9GB_CUDA_ERR;
   if (rc == T9GB_OK) {
      cudaGraph_t body = cp.conditional.phGraph_out[0];
      if (cudaStreamBeginCaptureToGraph(ctx->cap_stream, body, nullptr, nullptr, 0, cudaStreamCaptureModeThreadLocal)
         != cudaSuccess)
         rc = T9GB_CUDA_ERR;
      if (rc == T9GB_OK) {
         ctx->stream = ctx->cap_stream;
         rc = pcg_body(ctx, A, handle, 1);
         ctx->stream = s0;
         cudaGraph_t tmp = nullptr;
         if (cudaStreamEndCapture(ctx->cap_stream, &tmp) != cudaSuccess && rc == T9GB_OK)
            rc = T9GB_CUDA_ERR;
      }
   }
   if (rc == T9GB_OK)
      rc = pcg_finish(ctx, A);
   cudaError_t e = cudaStreamEndCapture(s0, &graph);
   if (rc == T9GB_OK && e != cudaSuccess) {
      ctx->last_error = std::string("graph capture: ") + cudaGetErrorString(e);
      rc = T9GB_CUDA_ERR;
   }
   if (rc == T9GB_OK) {
      e = cudaGraphInstantiate(&ctx->graph_exec[variant], graph, 0);
      if (e != cudaSuccess) {
         ctx->last_error = std::string("graph instantiate: ") + cudaGetErrorString(e);
         rc = T9GB_CUDA_ERR;
         ctx->graph_exec[variant] = nullptr;
      }
   }
   if (graph)
      cudaGraphDestroy(graph);
   cudaGetLastError();
   // the FFT plan was bound to the capture stream during the body
   cufftSetStream(ctx->pme.plan, ctx->stream);
   return rc;
}

static int induce_graph(Context* ctx, int variant)
{
   if (!ctx->graph_exec[variant])
      T9_CHECK(induce_capture(ctx, variant));
   T9_CHECK(list_request(ctx));
   T9_CUDA(cudaGraphLaunch(ctx->graph_exec[variant], ctx->stream));
   if (ctx->lx_k > 0)
      T9_CUDA(cudaEventRecord(ctx->ev_lx_fork, ctx->stream));
   if (ctx->stage_out)
      T9_CHECK(stage_dipoles(ctx));
   else if (ctx->out_d || ctx->out_p)
      T9_CHECK(scatter_from_sorted3(ctx, ctx->uind, ctx->out_d, ctx->out_p));
   if (ctx->after_launch && !ctx->after_done) {
      // the host waits for the solve only: the queued work runs on while it
      // reads the status and queues what follows
      T9_CUDA(cudaEventRecord(ctx->ev_solved, ctx->stream));
      T9_CHECK((*ctx->after_launch)());
      ctx->after_done = true;
      T9_CUDA(cudaEventSynchronize(ctx->ev_solved));
   } else {
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
   }
   ctx->list_stale = false;
   return T9GB_OK;
}

void drop_graphs(Context* ctx)
{
   for (auto& g : ctx->graph_exec)
      if (g) {
         cudaGraphExecDestroy(g);
         g = nullptr;
      }
}

// host policy for the start variant: compare both starts every learn_probe
// solves (and when the predictor history has just filled); in between start
// from what the last comparison chose for both systems
static int pick_variant_learn(Context* ctx)
{
   if (!(ctx->learn_mode & 2))
      return V_PLAIN;
   if (ctx->learn_since_probe >= ctx->learn_probe)
      return V_COMPARE;
   if (ctx->learn_last_choice == 3)
      return V_LEARNED;
   if (ctx->learn_last_choice == 0)
      return V_PLAIN;
   return V_COMPARE;
}

// the plain start with the predictor's ring full (as of the last solve)
// overlaps the guess's field with the permanent field (PME, the second grid)
static int pick_variant(Context* ctx)
{
   const int v = pick_variant_learn(ctx);
   if (v == V_PLAIN && ctx->learn_ring_full && pred_depth(ctx->cfg) > 0 && ctx->cfg.use_ewald && !ctx->prof.on &&
      (ctx->pcg_fuse & 8) && ctx->pme.qgrid2 != nullptr && ctx->side_stream[3] != nullptr)
      return V_PREDICT;
   return v;
}

static int lx_train_launch(Context* ctx, bool side);

int induce_sorted(Context* ctx)
{
   const bool graph = ctx->use_graph && !ctx->prof.on;
   const int variant = pick_variant(ctx);
   bool range_failed = false;
   ctx->induce_redone = false;
   T9_CHECK(lx_wait(ctx));
   for (int attempt = 0; attempt < 3; ++attempt) {
      if (attempt > 0)
         ctx->induce_redone = true;
      T9_CHECK(graph ? induce_graph(ctx, variant) : induce_stepwise(ctx, variant));
      int redo = 0;
      T9_CHECK(check_list_overflow(ctx, &redo));
      if (ctx->h_status[ST_RANGE]) {
         // a dipole-grid contribution reached the packed fixed-point guard:
         // widen the range (2^24 -> 2^16 scale) and solve again
         T9_CUDA(cudaMemsetAsync(ctx->status + ST_RANGE, 0, sizeof(int), ctx->stream));
         ctx->h_status[ST_RANGE] = 0;
         if (ctx->pme.pack_shift > 16) {
            ctx->pme.pack_shift = 16;
            drop_graphs(ctx);
            redo = 1;
         } else {
            range_failed = true;
         }
      }
      if (!redo)
         break;
      // the repeated solve saved a history frame: drop it
      if (pred_depth(ctx->cfg) > 0) {
         T9_CUDA(cudaMemcpy(ctx->h_status, ctx->status, sizeof(int) * ST_NSTAT, cudaMemcpyDeviceToHost));
         int v = ctx->h_status[ST_NUALT] - 1;
         T9_CUDA(cudaMemcpy(ctx->status + ST_NUALT, &v, sizeof(int), cudaMemcpyHostToDevice));
      }
   }
   if (!range_failed && ctx->h_status[ST_STATUS] == T9GB_OK)
      T9_CHECK(lx_train_launch(ctx, graph));
   prof_collect(ctx);
   ctx->last_iter = ctx->h_status[ST_ITER];
   ctx->last_eps = ctx->h_scal[S_EPS];
   ctx->last_status = ctx->h_status[ST_STATUS];
   if (range_failed) {
      ctx->last_error = "induced dipoles beyond the PME grid's fixed-point range (|alpha E| of order 10^3 e A)";
      ctx->last_status = T9GB_NAN_DETECTED;
   }
   ctx->learn_variant = variant;
   if (variant == V_COMPARE) {
      ctx->learn_last_choice = ctx->h_status[ST_LCHOICE];
      ctx->learn_since_probe = 1;
   } else {
      ctx->learn_since_probe += 1;
   }
   // the plain start changes character once the predictor history is full
   const bool full = pred_depth(ctx->cfg) > 0 && ctx->h_status[ST_NUALT] >= pred_depth(ctx->cfg);
   if (full != ctx->learn_ring_full)
      ctx->learn_since_probe = 1 << 30;
   ctx->learn_ring_full = full;
   return ctx->last_status;
}

// The fit of the solve just finished runs on its own stream, after the
// solve's graph (the converged frame is in the ring), beside what the host
// queues next; the next solve waits for it before it starts.  In the
// host-driven loop it runs in order.  Not after a failed solve.
static int lx_train_launch(Context* ctx, bool side)
{
   const int depth = pred_depth(ctx->cfg);
   if (ctx->lx_k <= 0 || ctx->lx_k >= depth)
      return T9GB_OK;
   const VecArgs A = vec_args(ctx);
   auto k = ctx->lx_k == 2 ? k_lx_train<2> : ctx->lx_k == 3 ? k_lx_train<3> : ctx->lx_k == 4 ? k_lx_train<4>
      : ctx->lx_k == 5 ? k_lx_train<5> : ctx->lx_k == 6 ? k_lx_train<6> : ctx->lx_k == 7 ? k_lx_train<7>
      : k_lx_train<8>;
   cudaStream_t st = ctx->stream;
   if (side) {
      T9_CUDA(cudaStreamWaitEvent(ctx->lx_stream, ctx->ev_lx_fork, 0));
      st = ctx->lx_stream;
   }
   k<<<LX_NB, 256, 0, st>>>(A, ctx->aspc_hist, ctx->lx_part, ctx->lx_ab, ctx->lx_coef_buf, ctx->status,
      ctx->lx_ticket, depth);
   T9_CUDA(cudaGetLastError());
   if (side) {
      T9_CUDA(cudaEventRecord(ctx->ev_lx_done, ctx->lx_stream));
      ctx->lx_pending = true;
   }
   return T9GB_OK;
}

// work on the ring and the coefficients waits for a fit still running
int lx_wait(Context* ctx)
{
   if (ctx->lx_pending) {
      T9_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_lx_done, 0));
      ctx->lx_pending = false;
   }
   return T9GB_OK;
}

// t9gb_learn_extrapolation: order 0 (the predictor's own coefficients) or
// 2 .. 8 ring frames (ASPC's ring of 16) / 2 .. 5 (Gear's ring of 6); every
// call starts a new fit
int lx_config(Context* ctx, int order)
{
   if (order != 0 && (order < 2 || order > LX_MAXK || order >= pred_depth(ctx->cfg)))
      return T9GB_BAD_ARG;
   T9_CHECK(lx_wait(ctx));
   if (order > 0 && !ctx->lx_ab) {
      T9_CUDA(cudaMalloc(&ctx->lx_ab, sizeof(double) * (LX_MAXK * LX_MAXK + LX_MAXK)));
      T9_CUDA(cudaMalloc(&ctx->lx_part, sizeof(float) * LX_NV * LX_NB));
      T9_CUDA(cudaMalloc(&ctx->lx_coef_buf, sizeof(float) * 16));
      T9_CUDA(cudaMalloc(&ctx->lx_ticket, sizeof(int)));
      T9_CUDA(cudaMemset(ctx->lx_ticket, 0, sizeof(int)));
      T9_CUDA(cudaStreamCreateWithFlags(&ctx->lx_stream, cudaStreamNonBlocking));
      T9_CUDA(cudaEventCreateWithFlags(&ctx->ev_lx_fork, cudaEventDisableTiming));
      T9_CUDA(cudaEventCreateWithFlags(&ctx->ev_lx_done, cudaEventDisableTiming));
   }
   if (ctx->lx_ab) {
      T9_CUDA(cudaMemsetAsync(ctx->lx_ab, 0, sizeof(double) * (LX_MAXK * LX_MAXK + LX_MAXK), ctx->stream));
      T9_CUDA(cudaMemsetAsync(ctx->lx_coef_buf, 0, sizeof(float) * 16, ctx->stream));
   }
   T9_CUDA(cudaMemsetAsync(ctx->status + ST_LX, 0, 2 * sizeof(int), ctx->stream));  // ST_LX, ST_LX_REJ
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   if (order != ctx->lx_k)
      drop_graphs(ctx);
   ctx->lx_k = order;
   ctx->lx_coef = order > 0 ? ctx->lx_coef_buf : nullptr;
   return T9GB_OK;
}

// t9gb_learn_extrapolation_state: after the fit of the last solve
int lx_state(Context* ctx, int* fits, int* rejected, float* coef16)
{
   int st[2] = {0, 0};
   float cf[16] = {};
   if (ctx->lx_k > 0) {
      T9_CHECK(lx_wait(ctx));
      T9_CUDA(cudaMemcpyAsync(st, ctx->status + ST_LX, sizeof(st), cudaMemcpyDeviceToHost, ctx->stream));
      T9_CUDA(cudaMemcpyAsync(cf, ctx->lx_coef_buf, sizeof(cf), cudaMemcpyDeviceToHost, ctx->stream));
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
   }
   if (fits)
      *fits = st[0];
   if (rejected)
      *rejected = st[1];
   if (coef16)
      for (int j = 0; j < 16; ++j)
         coef16[j] = cf[j];
   return T9GB_OK;
}

int reset_predictor(Context* ctx)
{
   T9_CHECK(lx_wait(ctx));
   ctx->learn_ring_full = false;
   T9_CUDA(cudaMemsetAsync(ctx->status + ST_NUALT, 0, sizeof(int), ctx->stream));
   return T9GB_OK;
}

// ---------------------------------------------------------------------------
// public field entry points (sorted internally, caller order at the boundary)

template <class F>
static int with_list(Context* ctx, F&& body)
{
   for (int attempt = 0; attempt < 3; ++attempt) {
      T9_CHECK(ensure_list(ctx));
      T9_CHECK(body());
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
      int redo = 0;
      T9_CHECK(check_list_overflow(ctx, &redo));
      int range = 0;
      T9_CUDA(cudaMemcpy(&range, ctx->status + ST_RANGE, sizeof(int), cudaMemcpyDeviceToHost));
      if (range) {
         T9_CUDA(cudaMemset(ctx->status + ST_RANGE, 0, sizeof(int)));
         if (ctx->pme.pack_shift <= 16) {
            ctx->last_error = "dipoles beyond the PME grid's fixed-point range";
            return T9GB_BAD_ARG;
         }
         ctx->pme.pack_shift = 16;
         drop_graphs(ctx);
         redo = 1;
      }
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
