// PME reciprocal-space field for AMOEBA: B-spline spreading of fractional
// multipoles or induced dipoles, convolution with the Ewald influence
// function, and the gather of potential derivatives fused with the
// reciprocal-self field terms.
//
// Reference pieces replaced (src/cu/pme.cu): gridPut_cu1<MPOLE> :14-183,
// gridPut_cu2<UIND> :185-255, fphiGet_cu<MPOLE/UIND2> :383-870, pmeConv_cu1
// :908-1031, cmpToFmp/cuindToFuind/fphiToCphi :1052-1300, and the recip-self
// kernels dfieldEwaldRecipSelfP2_cu1 / ufieldEwaldRecipSelfP1_cu1
// (src/cu/amoeba/field.cu:12-33, :71-118).
//
// Differences by design (same results up to rounding):
//  - the fractional transforms are folded into spread and gather (orthogonal
//    boxes: the transforms are diagonal);
//  - dfield and ufield only consume first derivatives of the potential, so the
//    gather evaluates 3 (MPOLE) or 6 (UIND) sums instead of 20 / 20;
//  - the influence function exp(-pi^2 h^2/a^2)/(pi V h^2 |b|^2) is tabulated
//    once per box (the reference recomputes it in every pmeConv call);
//  - the grid accumulates in 64-bit fixed point (order-independent), then one
//    pass converts it to the complex float grid and clears the fixed grid.
#include <cmath>
#include <utility>
#include <vector>

#include "common.cuh"
#include "reduce.cuh"

namespace t9gb {

// ---------------------------------------------------------------------------
// B-spline moduli |b(m)|^2 (Essmann et al., J. Chem. Phys. 103, 8577 (1995))
// with Tinker's optimal-zeta correction of Euler-spline zeros.

static void cardinal_bspline_knots(int order, double* c)
{
   const double x = 0;
   c[0] = 1 - x;
   c[1] = x;
   for (int k = 3; k <= order; ++k) {
      double denom = 1.0 / (k - 1);
      c[k - 1] = x * c[k - 2] * denom;
      for (int i = 1; i <= k - 2; ++i)
         c[k - i - 1] = ((x + i) * c[k - i - 2] + (k - i - x) * c[k - i - 1]) * denom;
      c[0] = (1 - x) * c[0] * denom;
   }
}

static void bspline_moduli(int nfft, int order, std::vector<double>& mod)
{
   const double pi = 3.14159265358979323846;
   std::vector<double> arr(nfft + order + 2, 0.0);
   double c[16];
   cardinal_bspline_knots(order, c);
   for (int i = 0; i < order; ++i)
      arr[i + 1] = c[i];
   mod.assign(nfft, 0.0);
   for (int i = 0; i < nfft; ++i) {
      double s1 = 0, s2 = 0;
      for (int j = 0; j < nfft; ++j) {
         double arg = 2 * pi * (double)i * (double)j / nfft;
         s1 += arr[j] * std::cos(arg);
         s2 += arr[j] * std::sin(arg);
      }
      mod[i] = s1 * s1 + s2 * s2;
   }
   const double eps = 1.0e-7;
   if (mod[0] < eps)
      mod[0] = 0.5 * mod[1];
   for (int i = 1; i < nfft - 1; ++i)
      if (mod[i] < eps)
         mod[i] = 0.5 * (mod[i - 1] + mod[i + 1]);
   if (mod[nfft - 1] < eps)
      mod[nfft - 1] = 0.5 * mod[nfft - 2];
   for (int i = 0; i < nfft; ++i) {
      int k = (i + 1 > nfft / 2) ? i - nfft : i;
      double zeta = 1;
      if (k != 0) {
         double s1 = 1, s2 = 1, f = pi * k / nfft;
         for (int j = 1; j <= 50; ++j) {
            double a1 = f / (f + pi * j), a2 = f / (f - pi * j);
            s1 += std::pow(a1, order) + std::pow(a2, order);
            s2 += std::pow(a1, 2 * order) + std::pow(a2, 2 * order);
         }
         zeta = s2 / s1;
      }
      mod[i] *= zeta * zeta;
   }
}

// ---------------------------------------------------------------------------
// per-site B-spline weights (include/seq/bsplgen.h:27-116), order 5

template <int LEVEL>
__device__ __forceinline__ void bspline5(float w, float th[5][LEVEL])
{
   float b[6][6];  // b[order][i], 1-based
   b[2][2] = w;
   b[2][1] = 1.f - w;
   b[3][3] = 0.5f * w * b[2][2];
   b[3][2] = 0.5f * ((1.f + w) * b[2][1] + (2.f - w) * b[2][2]);
   b[3][1] = 0.5f * (1.f - w) * b[2][1];
#pragma unroll
   for (int i = 4; i <= 5; ++i) {
      const int k = i - 1;
      const float denom = 1.f / k;
      b[i][i] = denom * w * b[k][k];
#pragma unroll
      for (int j = 1; j <= i - 2; ++j)
         b[i][i - j] = denom * ((w + j) * b[k][i - j - 1] + (i - j - w) * b[k][i - j]);
      b[i][1] = denom * (1.f - w) * b[k][1];
   }
   // derivative rows by repeated differencing of the lower-order rows
#pragma unroll
   for (int lv = 2; lv <= LEVEL; ++lv) {
      const int k = 5 - lv + 1;
#pragma unroll
      for (int pass = 0; pass < lv - 1; ++pass) {
         const int top = 5 - (lv - 2) + pass;
         b[k][top] = b[k][top - 1];
#pragma unroll
         for (int i = top - 1; i >= 2; --i)
            b[k][i] = b[k][i - 1] - b[k][i];
         b[k][1] = -b[k][1];
      }
   }
#pragma unroll
   for (int i = 1; i <= 5; ++i)
#pragma unroll
      for (int j = 1; j <= LEVEL; ++j)
         th[i - 1][j - 1] = b[5 - j + 1][i];
}

struct GridParams {
   int n1, n2, n3;
   float r1, r2, r3;  // 1/box
   float a1, a2, a3;  // nfft / box
   float selfterm;    // 4 a^3 / (3 sqrt(pi))
   float pk_s, pk_lim;  // dipole grids: 32-bit fixed-point scale, per-contribution guard
   int* range;          // set when a contribution reaches pk_lim
};

__device__ __forceinline__ void site(const GridParams& G, float4 p, int& i1, int& i2, int& i3, float& w1, float& w2,
   float& w3)
{
   float w = p.x * G.r1;
   w = w + 0.5f - floorf(w + 0.5f);
   float fr = G.n1 * w;
   i1 = (int)floorf(fr);
   w1 = fr - i1;
   w = p.y * G.r2;
   w = w + 0.5f - floorf(w + 0.5f);
   fr = G.n2 * w;
   i2 = (int)floorf(fr);
   w2 = fr - i2;
   w = p.z * G.r3;
   w = w + 0.5f - floorf(w + 0.5f);
   fr = G.n3 * w;
   i3 = (int)floorf(fr);
   w3 = fr - i3;
   i1 -= BSORDER - 1;
   i2 -= BSORDER - 1;
   i3 -= BSORDER - 1;
   i1 += (i1 < 0 ? G.n1 : 0);
   i2 += (i2 < 0 ? G.n2 : 0);
   i3 += (i3 < 0 ? G.n3 : 0);
}

// Fixed-point grid: one 64-bit word per point.  Multipole grids hold the
// real part at scale 2^40 (to_fx).  Dipole grids pack the d value (high 32
// bits) and the p value (low 32 bits) as 32-bit fixed point at scale pk_s
// (2^24, or 2^16 after a range fallback): the word sum is A 2^32 + B for the
// sums A, B of the halves, and both are recovered exactly while each stays
// within the signed 32-bit range, so one reduction carries both grids.

// fire-and-forget 64-bit reduction (no value returned, so the warp does not
// wait on it)
__device__ __forceinline__ void red_u64(unsigned long long* q, size_t idx, unsigned long long v)
{
   asm volatile("red.global.add.u64 [%0], %1;" ::"l"(q + idx), "l"(v) : "memory");
}

__device__ __forceinline__ void grid_add(unsigned long long* q, size_t idx, float v)
{
   if (v != 0.f)
      red_u64(q, idx, (unsigned long long)to_fx(v));
}

// d and p values of one point into one word; a value at or above pk_lim in
// magnitude (1/32 of the half's range) raises the range flag
__device__ __forceinline__ void grid_add2(unsigned long long* q, size_t idx, float vd, float vp, const GridParams& G)
{
   if (vd == 0.f && vp == 0.f)
      return;
   if (!(fabsf(vd) < G.pk_lim && fabsf(vp) < G.pk_lim)) {
      atomicOr(G.range, 1);
      return;
   }
   const long long a = __float2int_rn(vd * G.pk_s), b = __float2int_rn(vp * G.pk_s);
   red_u64(q, idx, (unsigned long long)(a * 4294967296ll + b));
}

// one word of the fixed-point grid as a complex value
__device__ __forceinline__ float2 grid_word(long long w, int packed, float inv)
{
   if (!packed)
      return make_float2(from_fx(w), 0.f);
   const int b = (int)(unsigned)(unsigned long long)w;
   const int a = (int)((w - (long long)b) >> 32);
   return make_float2((float)a * inv, (float)b * inv);
}

// the guard on the sums of a packed word: each contribution stays below
// 2^26, so a half at or above 2^30 in magnitude (16 or more near-limit
// contributions of one sign, far beyond real grids) is taken as a sum that
// may have left the 32-bit range, and the solve is repeated at the wider
// scale, as for a large contribution
__device__ __forceinline__ bool grid_word_big(long long w, int packed)
{
   if (!packed)
      return false;
   const int b = (int)(unsigned)(unsigned long long)w;
   const int a = (int)((w - (long long)b) >> 32);
   return a >= (1 << 30) || a <= -(1 << 30) || b >= (1 << 30) || b <= -(1 << 30);
}

// Spreading, one warp per atom: lane (jy, kz) < 25 owns one row of five x
// points.  MODE 0 spreads fractional multipoles into the real part; MODE 1
// spreads fractional d dipoles into the real and p dipoles into the
// imaginary part.  rp rows are 12 floats (q, d, quadrupole, ...), u rows 8.
// DIR (MODE 1): the dipoles are the CG search direction p = z + b p_old
// (src = p_old, z8 = z, b from scal), formed as each row is read.
template <int MODE, bool DIR = false>
__global__ void __launch_bounds__(256) k_spread(int n, GridParams G, const float4* __restrict__ spos,
   const float* __restrict__ src, const float* __restrict__ z8, const double* __restrict__ scal,
   unsigned long long* __restrict__ q)
{
   // the site and the B-splines need the positions only: they are formed
   // before the wait for the programmatic predecessor (no-op otherwise)
   const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int lane = threadIdx.x & 31;
   if (s >= n || lane >= 25)
      return;
   int i1, i2, i3;
   float w1, w2, w3;
   site(G, spos[s], i1, i2, i3, w1, w2, w3);
   constexpr int L = MODE == 0 ? 3 : 2;
   float t1[5][L], t2[5][L], t3[5][L];
   bspline5<L>(w1, t1);
   bspline5<L>(w2, t2);
   bspline5<L>(w3, t3);
   pdl_wait();
   pdl_trigger();
   const int jy = lane % 5, kz = lane / 5;
   int zb = i3 + kz;
   zb -= (zb >= G.n3 ? G.n3 : 0);
   int yb = i2 + jy;
   yb -= (yb >= G.n2 ? G.n2 : 0);
   const size_t row = ((size_t)zb * G.n2 + yb) * G.n1;
   const float v0 = t3[kz][0], v1 = t3[kz][1];
   const float u0 = t2[jy][0], u1 = t2[jy][1];
   if (MODE == 0) {
      const float* m = src + 12 * s;
      // Cartesian -> fractional (orthogonal box; quadrupole off-diagonals doubled)
      const float f0 = m[0];
      const float fx = G.a1 * m[1], fy = G.a2 * m[2], fz = G.a3 * m[3];
      const float fxx = G.a1 * G.a1 * m[4], fyy = G.a2 * G.a2 * m[5], fzz = G.a3 * G.a3 * m[6];
      const float fxy = 2.f * G.a1 * G.a2 * m[7], fxz = 2.f * G.a1 * G.a3 * m[8], fyz = 2.f * G.a2 * G.a3 * m[9];
      const float v2 = t3[kz][L - 1], u2 = t2[jy][L - 1];
      const float term0 = f0 * u0 * v0 + fy * u1 * v0 + fz * u0 * v1 + fyy * u2 * v0 + fzz * u0 * v2 + fyz * u1 * v1;
      const float term1 = fx * u0 * v0 + fxy * u1 * v0 + fxz * u0 * v1;
      const float term2 = fxx * u0 * v0;
#pragma unroll
      for (int ix = 0; ix < 5; ++ix) {
         int xb = i1 + ix;
         xb -= (xb >= G.n1 ? G.n1 : 0);
         grid_add(q, row + xb, term0 * t1[ix][0] + term1 * t1[ix][1] + term2 * t1[ix][L - 1]);
      }
   } else {
      float u[8];
      if (DIR)
         dir_row(src, z8, s, (float)scal[S_B_D], (float)scal[S_B_P], u);
      else
#pragma unroll
         for (int c = 0; c < 6; ++c)
            u[c] = src[8 * s + c];
      const float dx = G.a1 * u[0], dy = G.a2 * u[1], dz = G.a3 * u[2];
      const float px = G.a1 * u[3], py = G.a2 * u[4], pz = G.a3 * u[5];
      const float d01 = dy * u1 * v0 + dz * u0 * v1, d11 = dx * u0 * v0;
      const float p01 = py * u1 * v0 + pz * u0 * v1, p11 = px * u0 * v0;
#pragma unroll
      for (int ix = 0; ix < 5; ++ix) {
         int xb = i1 + ix;
         xb -= (xb >= G.n1 ? G.n1 : 0);
         grid_add2(q, row + xb, d01 * t1[ix][0] + d11 * t1[ix][1], p01 * t1[ix][0] + p11 * t1[ix][1], G);
      }
   }
}

// fixed -> complex float, clearing the fixed grid for the next spread
__global__ void k_fx_to_grid(size_t ng, long long* __restrict__ q, float2* __restrict__ g, int packed, float inv,
   int* __restrict__ range)
{
   bool big = false;
   for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ng; i += (size_t)gridDim.x * blockDim.x) {
      const long long w = q[i];
      big |= grid_word_big(w, packed);
      g[i] = grid_word(w, packed, inv);
      q[i] = 0;
   }
   if (big)
      atomicOr(range, 1);
}

// reciprocal convolution with the tabulated influence function
__global__ void k_conv(size_t ng, const float* __restrict__ infl, float2* __restrict__ g)
{
   for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ng; i += (size_t)gridDim.x * blockDim.x) {
      float2 v = g[i];
      float f = infl[i];
      g[i] = make_float2(v.x * f, v.y * f);
   }
}

// Gather of the first potential derivatives fused with the recip + self
// field, one warp per atom: lane (jy, kz) < 25 reads one row of five points,
// a fixed xor tree combines the rows.  MODE 0: real part -> d and p field,
// self term with the permanent dipole.  MODE 1: real -> d, imaginary -> p,
// self term with the induced dipoles.  Plain stores, rows of 8 floats.
// AP (MODE 1, ACC): the dipoles are the CG search direction p = z + b p_old
// (P.conj = p_old, P.zrsd = z); instead of the field, lane 0 stores
// p and Ap = p/alpha - field, and the block partials of p.Ap give, in the
// last block, the step length a = s / p.Ap.  Atoms are visited warp-strided
// over at most RED_MAX blocks.
// LATE: the kernel has not waited for its programmatic predecessor yet; the
// site and the B-splines (positions only) are formed first, then the wait,
// then the grid and dipole reads, so the prologue overlaps the predecessor.
template <int MODE, bool ACC, bool AP, bool DIR, bool LATE = false>
__device__ __forceinline__ void gather_atom(int s, int lane, const GridParams& G, const float4* __restrict__ spos,
   const float2* __restrict__ g, const float* __restrict__ rp, const float* __restrict__ u8, float* __restrict__ out,
   const PcgAp& P, float bd, float bp, float* pap)
{
   int i1, i2, i3;
   float w1, w2, w3;
   site(G, spos[s], i1, i2, i3, w1, w2, w3);
   float acc[6] = {0, 0, 0, 0, 0, 0};
   float t1[5][2], t2[5][2], t3[5][2];
   bspline5<2>(w1, t1);
   bspline5<2>(w2, t2);
   bspline5<2>(w3, t3);
   if (LATE)
      pdl_wait();
   if (lane < 25) {
      const int jy = lane % 5, kz = lane / 5;
      int zb = i3 + kz;
      zb -= (zb >= G.n3 ? G.n3 : 0);
      int yb = i2 + jy;
      yb -= (yb >= G.n2 ? G.n2 : 0);
      const size_t row = ((size_t)zb * G.n2 + yb) * G.n1;
      float rt0 = 0.f, rt1 = 0.f, it0 = 0.f, it1 = 0.f;
#pragma unroll
      for (int ix = 0; ix < 5; ++ix) {
         int xb = i1 + ix;
         xb -= (xb >= G.n1 ? G.n1 : 0);
         const float2 qv = g[row + xb];
         rt0 += qv.x * t1[ix][0];
         rt1 += qv.x * t1[ix][1];
         if (MODE == 1) {
            it0 += qv.y * t1[ix][0];
            it1 += qv.y * t1[ix][1];
         }
      }
      const float u0 = t2[jy][0], u1 = t2[jy][1], v0 = t3[kz][0], v1 = t3[kz][1];
      acc[0] = rt1 * u0 * v0;
      acc[1] = rt0 * u1 * v0;
      acc[2] = rt0 * u0 * v1;
      if (MODE == 1) {
         acc[3] = it1 * u0 * v0;
         acc[4] = it0 * u1 * v0;
         acc[5] = it0 * u0 * v1;
      }
   }
#pragma unroll
   for (int c = 0; c < (MODE == 1 ? 6 : 3); ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
   if (AP) {
      // lane c < 6 finishes component c: p, its recip + self field added to
      // the real-space field, Ap = p/alpha - field, and p.Ap
      if (lane < 6) {
         float ac = acc[0];
#pragma unroll
         for (int k = 1; k < 6; ++k)
            if (lane == k)
               ac = acc[k];
         const int c = lane, x = 8 * s + c;
         const float gc = c % 3 == 0 ? G.a1 : (c % 3 == 1 ? G.a2 : G.a3);
         const float p = __fmaf_rn(c < 3 ? bd : bp, P.conj[x], P.zrsd[x]);
         const float fld = out[x] + (G.selfterm * p - gc * ac);
         const float v = P.polinv[s] * p - fld;
         P.vec[x] = v;
         P.conj[x] = p;
         pap[c < 3 ? 0 : 1] += p * v;
      }
      return;
   }
   if (lane != 0)
      return;
   float* a = out + 8 * s;
   float r[6];
   if (MODE == 0) {
      const float* m = rp + 12 * s;
      r[0] = r[3] = -G.a1 * acc[0] + G.selfterm * m[1];
      r[1] = r[4] = -G.a2 * acc[1] + G.selfterm * m[2];
      r[2] = r[5] = -G.a3 * acc[2] + G.selfterm * m[3];
   } else {
      float u[8];
      if (DIR)
         dir_row(P.conj, P.zrsd, s, bd, bp, u);
      else
#pragma unroll
         for (int c = 0; c < 6; ++c)
            u[c] = u8[8 * s + c];
      r[0] = G.selfterm * u[0] - G.a1 * acc[0];
      r[1] = G.selfterm * u[1] - G.a2 * acc[1];
      r[2] = G.selfterm * u[2] - G.a3 * acc[2];
      r[3] = G.selfterm * u[3] - G.a1 * acc[3];
      r[4] = G.selfterm * u[4] - G.a2 * acc[4];
      r[5] = G.selfterm * u[5] - G.a3 * acc[5];
   }
   // ACC: add to the real-space field already stored (the same two-operand
   // sum the real-space kernel forms when it adds this result as its base)
#pragma unroll
   for (int c = 0; c < 6; ++c)
      a[c] = ACC ? a[c] + r[c] : r[c];
}

template <int MODE, bool ACC, bool AP = false, bool DIR = false>
__global__ void __launch_bounds__(256, 6) k_gather_field(int n, GridParams G, const float4* __restrict__ spos,
   const float2* __restrict__ g, const float* __restrict__ rp, const float* __restrict__ u8, float* __restrict__ out,
   PcgAp P)
{
   // the plain gather waits inside gather_atom, after its position-only prologue
   constexpr bool LATE = !AP && !DIR;
   if (!LATE)
      pdl_wait();
   const int lane = threadIdx.x & 31;
   if (!AP) {
      const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
      float bd = 0.f, bp = 0.f;
      if (DIR) {
         bd = (float)P.scal[S_B_D];
         bp = (float)P.scal[S_B_P];
      }
      if (s < n)
         gather_atom<MODE, ACC, false, DIR, LATE>(s, lane, G, spos, g, rp, u8, out, P, bd, bp, nullptr);
      else if (LATE)
         pdl_wait();
      return;
   }
   __shared__ double sh[64];
   const float bd = (float)P.scal[S_B_D], bp = (float)P.scal[S_B_P];
   float pap[2] = {0.f, 0.f};
   const int nw = (gridDim.x * blockDim.x) >> 5;
   for (int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; s < n; s += nw)
      gather_atom<MODE, ACC, true, false>(s, lane, G, spos, g, rp, u8, out, P, bd, bp, pap);
   store_partials_f<2>(P.red, R_PAP_D, pap, sh);
   if (!last_block(P.state + ST_TICKET1))
      return;
   double tot[2];
   sum_slots(P.red, R_PAP_D, 2, gridDim.x, sh, tot);
   if (threadIdx.x == 0) {  // the step lengths in FP32 (used as FP32)
      P.scal[S_A_D] = tot[0] == 0 ? 0.0 : (double)((float)P.scal[S_SUM_D] / (float)tot[0]);
      P.scal[S_A_P] = tot[1] == 0 ? 0.0 : (double)((float)P.scal[S_SUM_P] / (float)tot[1]);
   }
}

// Multipole reciprocal + self energy per atom (warp per atom, level-3
// weights): e = 1/2 f sum_k fmp_k fphi_k (src/cu/hippo/empole.cu:202-335)
// and the Ewald self energy (include/seq/emselfamoeba.h:7-37), stored per
// atom in e_atom[s] and e_self[s].
__global__ void __launch_bounds__(256) k_empole_recip_self(int n, GridParams G, float f, float aewald,
   const float4* __restrict__ spos, const float2* __restrict__ g, const float* __restrict__ rp,
   double* __restrict__ e_atom, double* __restrict__ e_self)
{
   const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int lane = threadIdx.x & 31;
   if (s >= n)
      return;
   int i1, i2, i3;
   float w1, w2, w3;
   site(G, spos[s], i1, i2, i3, w1, w2, w3);
   float phi[10] = {0, 0, 0, 0, 0, 0, 0, 0, 0, 0};
   if (lane < 25) {
      float t1[5][3], t2[5][3], t3[5][3];
      bspline5<3>(w1, t1);
      bspline5<3>(w2, t2);
      bspline5<3>(w3, t3);
      const int jy = lane % 5, kz = lane / 5;
      int zb = i3 + kz;
      zb -= (zb >= G.n3 ? G.n3 : 0);
      int yb = i2 + jy;
      yb -= (yb >= G.n2 ? G.n2 : 0);
      const size_t row = ((size_t)zb * G.n2 + yb) * G.n1;
      float t0 = 0.f, ta = 0.f, tb = 0.f;
#pragma unroll
      for (int ix = 0; ix < 5; ++ix) {
         int xb = i1 + ix;
         xb -= (xb >= G.n1 ? G.n1 : 0);
         const float q = g[row + xb].x;
         t0 += q * t1[ix][0];
         ta += q * t1[ix][1];
         tb += q * t1[ix][2];
      }
      const float u0 = t2[jy][0], u1 = t2[jy][1], u2 = t2[jy][2];
      const float v0 = t3[kz][0], v1 = t3[kz][1], v2 = t3[kz][2];
      phi[0] = t0 * u0 * v0;
      phi[1] = ta * u0 * v0;
      phi[2] = t0 * u1 * v0;
      phi[3] = t0 * u0 * v1;
      phi[4] = tb * u0 * v0;
      phi[5] = t0 * u2 * v0;
      phi[6] = t0 * u0 * v2;
      phi[7] = ta * u1 * v0;
      phi[8] = ta * u0 * v1;
      phi[9] = t0 * u1 * v1;
   }
#pragma unroll
   for (int c = 0; c < 10; ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         phi[c] += __shfl_xor_sync(0xffffffffu, phi[c], o);
   if (lane != 0)
      return;
   const float* m = rp + 12 * s;
   const double fmp[10] = {m[0], G.a1 * m[1], G.a2 * m[2], G.a3 * m[3], G.a1 * G.a1 * m[4], G.a2 * G.a2 * m[5],
      G.a3 * G.a3 * m[6], 2.f * G.a1 * G.a2 * m[7], 2.f * G.a1 * G.a3 * m[8], 2.f * G.a2 * G.a3 * m[9]};
   double e = 0;
   for (int c = 0; c < 10; ++c)
      e += fmp[c] * (double)phi[c];
   e_atom[s] = 0.5 * f * e;
   const double a2 = 2.0 * aewald * aewald;
   const double fterm = -(double)f * aewald / 1.77245385090551602730;
   const double cii = (double)m[0] * m[0];
   const double dii = (double)m[1] * m[1] + (double)m[2] * m[2] + (double)m[3] * m[3];
   const double qii = 2.0 * ((double)m[7] * m[7] + (double)m[8] * m[8] + (double)m[9] * m[9]) + (double)m[4] * m[4]
      + (double)m[5] * m[5] + (double)m[6] * m[6];
   e_self[s] = fterm * (cii + a2 * (dii / 3.0 + 2.0 * a2 * qii * 0.2));
}

// ---------------------------------------------------------------------------
// Fused 3-D FFT + convolution for cubic power-of-two grids (N = 32, 64, 128
// points per edge), replacing cuFFT's six kernels plus the fixed-point
// conversion and the convolution of one pass by three kernels:
//   k_fft_plane<FROM_FX, forward>: fixed-point grid -> float (the fixed-point
//     grid is cleared for the next spread), 2-D forward FFT of each z plane;
//   k_fft_zline<MODE 2>: forward FFT along z, times the influence function,
//     inverse FFT along z, for 16 x-adjacent lines per block (the virial path
//     splits it into MODE 0 forward / MODE 1 inverse around the k-space pass);
//   k_fft_plane<inverse>: 2-D inverse FFT of each plane.
// A line transform of N = N1 x T points runs on T threads (8; 4 for N = 32)
// of one warp, each holding N1 points in registers: an N1-point DFT over the
// stride-T subsequence, the twiddle W_N^(t k1), an exchange through shared
// memory, then N1 / T T-point DFTs per thread (Cooley-Tukey with
// n = n1 T + n2, k = k1 + N1 k2).  Forward e^{-2 pi i k n / N}, inverse
// unnormalised, as cuFFT's C2C; the twiddles come from a table computed in
// double precision.

__constant__ float2 c_tw[128];  // e^{-2 pi i k / 128}

__device__ __forceinline__ float2 cmulf(float2 a, float2 b)
{
   return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}

__host__ __device__ constexpr int brev_c(int x, int bits)
{
   int r = 0;
   for (int b = 0; b < bits; ++b) {
      r = (r << 1) | (x & 1);
      x >>= 1;
   }
   return r;
}

__host__ __device__ constexpr int log2_c(int m) { return m <= 1 ? 0 : 1 + log2_c(m / 2); }

// in-register M-point DFT (M = 4, 8, 16), natural order in and out;
// tw: e^{-2 pi i k / 128} in shared memory (uniform indices: broadcasts)
template <int M, bool INV>
__device__ __forceinline__ void dft_reg(float2* v, const float2* tw)
{
   constexpr int L = log2_c(M);
#pragma unroll
   for (int i = 0; i < M; ++i) {
      const int j = brev_c(i, L);
      if (j > i) {
         const float2 a = v[i];
         v[i] = v[j];
         v[j] = a;
      }
   }
#pragma unroll
   for (int st = 1; st <= L; ++st) {
      const int len = 1 << st, half = len / 2, step = 128 / len;
#pragma unroll
      for (int b = 0; b < M; b += len)
#pragma unroll
         for (int k = 0; k < half; ++k) {
            float2 w = tw[k * step];
            if (INV)
               w.y = -w.y;
            const float2 a = v[b + k];
            const float2 c = k == 0 ? v[b + k + half] : cmulf(w, v[b + k + half]);
            v[b + k] = make_float2(a.x + c.x, a.y + c.y);
            v[b + k + half] = make_float2(a.x - c.x, a.y - c.y);
         }
   }
}

// Shared-memory swizzle of a line index: the low bits within each block of T
// are XORed with the block number (and the block group), so the strided
// step-2 reads of fft_line and the column passes spread over the banks.
template <int T>
__device__ __forceinline__ int fsig(int i)
{
   return i ^ (((i / T) + (i / (T * T))) & (T - 1));
}

// One N-point line, element i at line[fsig(i) * ls], transformed in place by
// the T threads t = 0..T-1 of one warp (every thread of the warp takes part
// in some line).
// wt[k1] = W_N^(t k1) for this thread's t, read once per kernel from the
// table (its thread-dependent indices would conflict on every line).
template <int N, int T>
__device__ __forceinline__ void fft_twiddles(int t, const float2* tw, float2* wt)
{
   if (N / T <= 8) {
#pragma unroll
      for (int k1 = 0; k1 < N / T; ++k1)
         wt[k1] = tw[((t * k1) & (N - 1)) * (128 / N)];
   }
}

template <int N, int T, bool INV>
__device__ __forceinline__ void fft_line(float2* line, int ls, int t, const float2* tw, const float2* wt)
{
   constexpr int N1 = N / T, J = N1 / T;
   float2 v[N1];
#pragma unroll
   for (int n1 = 0; n1 < N1; ++n1)
      v[n1] = line[fsig<T>(n1 * T + t) * ls];
   dft_reg<N1, INV>(v, tw);
#pragma unroll
   for (int k1 = 1; k1 < N1; ++k1) {
      // registers for up to 8 twiddles; the 128-point lines (1024-thread
      // planes) read the table rather than spill
      float2 w = N1 <= 8 ? wt[k1] : tw[((t * k1) & (N - 1)) * (128 / N)];
      if (INV)
         w.y = -w.y;
      v[k1] = cmulf(v[k1], w);
   }
   __syncwarp();
#pragma unroll
   for (int k1 = 0; k1 < N1; ++k1)
      line[fsig<T>(k1 * T + t) * ls] = v[k1];
   __syncwarp();
   float2 u[J][T];
#pragma unroll
   for (int j = 0; j < J; ++j) {
      const int k1 = t * J + j;
#pragma unroll
      for (int n2 = 0; n2 < T; ++n2)
         u[j][n2] = line[fsig<T>(k1 * T + n2) * ls];
      dft_reg<T, INV>(u[j], tw);
   }
   __syncwarp();
#pragma unroll
   for (int j = 0; j < J; ++j)
#pragma unroll
      for (int k2 = 0; k2 < T; ++k2)
         line[fsig<T>(t * J + j + N1 * k2) * ls] = u[j][k2];
   __syncwarp();
}

template <int N>
__host__ __device__ constexpr int fft_threads_per_line()
{
   return N == 32 ? 4 : 8;
}

// row pitch of the plane (float2) and of the z-line tile
template <int N>
__host__ __device__ constexpr int fft_plane_ld()
{
   return N == 32 ? N + 4 : N + 2;
}

template <int N>
__host__ __device__ constexpr int fft_zline_ld()
{
   return N == 32 ? 20 : 18;
}

// 2-D FFT (x then y) of z plane blockIdx.x; N * T threads, dynamic shared
// memory N (N + 1) + 128 float2
template <int N, bool FROM_FX, bool INV>
__global__ void __launch_bounds__(N * fft_threads_per_line<N>()) k_fft_plane(long long* __restrict__ qfx,
   float2* __restrict__ g, int packed, float inv, int* __restrict__ range)
{
   pdl_wait();
   pdl_trigger();  // the next kernel may stage its blocks and run its prologue
   // element (y, x) at fsm[fsig(y) LD + fsig(x)]; the padding keeps the two
   // lines of a 16-thread shared-memory phase on different banks
   constexpr int T = fft_threads_per_line<N>(), LD = fft_plane_ld<N>(), NT = N * T, R = N / T;
   extern __shared__ float2 fsm[];
   float2* tw = fsm + N * LD;
   for (int k = threadIdx.x; k < 128; k += NT)
      tw[k] = c_tw[k];
   const size_t base = (size_t)blockIdx.x * N * N;
   // element e = threadIdx.x + r NT, r < R: all loads of a chunk in flight together
   bool big = false;
#pragma unroll
   for (int c = 0; c < R; c += 8) {
      float2 v[8];
      if (FROM_FX) {
         long long* q = qfx + base + threadIdx.x;
         long long f[8];
#pragma unroll
         for (int r = 0; r < 8; ++r)
            f[r] = q[(c + r) * NT];
#pragma unroll
         for (int r = 0; r < 8; ++r) {
            q[(c + r) * NT] = 0;
            big |= grid_word_big(f[r], packed);
            v[r] = grid_word(f[r], packed, inv);
         }
      } else {
#pragma unroll
         for (int r = 0; r < 8; ++r)
            v[r] = g[base + threadIdx.x + (c + r) * NT];
      }
#pragma unroll
      for (int r = 0; r < 8; ++r) {
         const int e = threadIdx.x + (c + r) * NT;
         fsm[fsig<T>(e / N) * LD + fsig<T>(e % N)] = v[r];
      }
   }
   if (FROM_FX && big)
      atomicOr(range, 1);
   __syncthreads();
   const int line = threadIdx.x / T, t = threadIdx.x % T;
   float2 wt[N / T];
   fft_twiddles<N, T>(t, tw, wt);
   fft_line<N, T, INV>(fsm + fsig<T>(line) * LD, 1, t, tw, wt);  // row y = line, along x
   __syncthreads();
   fft_line<N, T, INV>(fsm + fsig<T>(line), LD, t, tw, wt);  // column x = line, along y
   __syncthreads();
#pragma unroll
   for (int r = 0; r < R; ++r) {
      const int e = threadIdx.x + r * NT;
      g[base + e] = fsm[fsig<T>(e / N) * LD + fsig<T>(e % N)];
   }
}

// Lines along z of 16 adjacent x at one y.  MODE 0 forward, 1 inverse,
// 2 forward, influence function, inverse.
template <int N, int MODE>
__global__ void __launch_bounds__(16 * fft_threads_per_line<N>()) k_fft_zline(const float* __restrict__ infl,
   float2* __restrict__ g)
{
   pdl_wait();
   pdl_trigger();  // the next kernel may stage its blocks and run its prologue
   // element z of line l at sm[fsig(z) LD + l]
   constexpr int T = fft_threads_per_line<N>(), XL = 16, LD = fft_zline_ld<N>(), NT = XL * T, R = N / T;
   __shared__ float2 sm[N * LD];
   __shared__ float2 tw[128];
   for (int k = threadIdx.x; k < 128; k += NT)
      tw[k] = c_tw[k];
   const int xb = (blockIdx.x % (N / XL)) * XL, y = blockIdx.x / (N / XL);
   const size_t base = (size_t)y * N + xb, zs = (size_t)N * N;
   // element e = threadIdx.x + r NT of the [z][16] tile: z = e / 16, x = e % 16
   const int ex = threadIdx.x % XL, ez = threadIdx.x / XL;
   constexpr int ZS = NT / XL;  // z rows per r step
#pragma unroll
   for (int c = 0; c < R; c += 8) {
      float2 v[8];
#pragma unroll
      for (int r = 0; r < 8; ++r)
         v[r] = g[base + (size_t)(ez + (c + r) * ZS) * zs + ex];
#pragma unroll
      for (int r = 0; r < 8; ++r)
         sm[fsig<T>(ez + (c + r) * ZS) * LD + ex] = v[r];
   }
   __syncthreads();
   const int line = threadIdx.x / T, t = threadIdx.x % T;
   float2 wt[N / T];
   fft_twiddles<N, T>(t, tw, wt);
   if (MODE != 1)
      fft_line<N, T, false>(sm + line, LD, t, tw, wt);
   if (MODE == 2) {
      __syncthreads();
#pragma unroll
      for (int c = 0; c < R; c += 8) {
         float f[8];
#pragma unroll
         for (int r = 0; r < 8; ++r)
            f[r] = infl[base + (size_t)(ez + (c + r) * ZS) * zs + ex];
#pragma unroll
         for (int r = 0; r < 8; ++r) {
            float2& v = sm[fsig<T>(ez + (c + r) * ZS) * LD + ex];
            v = make_float2(v.x * f[r], v.y * f[r]);
         }
      }
      __syncthreads();
   }
   if (MODE != 0)
      fft_line<N, T, true>(sm + line, LD, t, tw, wt);
   __syncthreads();
#pragma unroll
   for (int r = 0; r < R; ++r)
      g[base + (size_t)(ez + r * ZS) * zs + ex] = sm[fsig<T>(ez + r * ZS) * LD + ex];
}

// ---------------------------------------------------------------------------
// The same 2-D plane transform spread over a thread-block cluster of CL CTAs
// per z plane (N CL CTAs in all).  CTA r of the cluster stages rows
// [r R, r R + R) of the plane (R = N / CL), one contiguous R N-word slab,
// with one bulk asynchronous copy (cp.async.bulk, completion on an mbarrier
// with a bounded wait), transforms them along x, and after a cluster barrier
// gathers columns [r R, r R + R) of the whole plane from the R-row tiles of
// the CL CTAs through distributed shared memory; it transforms those along y
// and stores them.  The per-line arithmetic is fft_line's, in the same order
// as k_fft_plane, so the results are bit-identical to it.
template <int N, int CL>
struct PlaneCl {
   static constexpr int T = fft_threads_per_line<N>();
   static constexpr int R = N / CL;           // rows (and columns) per CTA
   static constexpr int NT = R * T;           // threads
   static constexpr int LDR = N + 2;          // row tile pitch (float2)
   static constexpr int LDC = R + 1;          // column tile pitch
   static constexpr int PER = R * N / NT;     // elements per thread in a tile copy
   static constexpr size_t STAGE = (size_t)R * N * 8;  // bytes of the staged slab
   static constexpr size_t SMEM = STAGE + sizeof(float2) * ((size_t)R * LDR + (size_t)N * LDC + 128) + 16;
};

template <int N, int CL, bool FROM_FX, bool INV>
__global__ void __launch_bounds__(PlaneCl<N, CL>::NT) k_fft_plane_cl(long long* __restrict__ qfx,
   float2* __restrict__ g, int packed, float inv, int* __restrict__ err)
{
   using C = PlaneCl<N, CL>;
   constexpr int T = C::T, R = C::R, NT = C::NT, LDR = C::LDR, LDC = C::LDC, PER = C::PER;
   extern __shared__ __align__(128) unsigned char smem_raw[];
   unsigned long long* stage = reinterpret_cast<unsigned long long*>(smem_raw);
   float2* rowt = reinterpret_cast<float2*>(smem_raw + C::STAGE);
   float2* colt = rowt + R * LDR;
   float2* tw = colt + N * LDC;
   unsigned long long* bar = reinterpret_cast<unsigned long long*>(tw + 128);
   unsigned rank;
   asm volatile("mov.u32 %0, %%cluster_ctarank;" : "=r"(rank));
   const int z = blockIdx.x / CL;
   const size_t base = (size_t)z * N * N + (size_t)rank * R * N;  // first word of this CTA's rows
   const unsigned bar_s = (unsigned)__cvta_generic_to_shared(bar);
   const unsigned stage_s = (unsigned)__cvta_generic_to_shared(stage);
   if (threadIdx.x == 0)
      mbar_init(bar_s, 1);
   __syncthreads();
   if (threadIdx.x == 0) {
      const void* src = FROM_FX ? static_cast<const void*>(qfx + base) : static_cast<const void*>(g + base);
      mbar_expect_tx(bar_s, (unsigned)C::STAGE);
      bulk_g2s(stage_s, src, (unsigned)C::STAGE, bar_s);
   }
   for (int k = threadIdx.x; k < 128; k += NT)
      tw[k] = c_tw[k];
   if (!mbar_wait_bounded(bar_s, 0)) {
      // the copy never completed: record it, wait once more for it, go on
      if (threadIdx.x == 0)
         atomicExch(err, 1);
      mbar_wait_bounded(bar_s, 0);
   }
   // staged slab -> row tile (element e: row e / N, column e % N)
#pragma unroll
   for (int k = 0; k < PER; ++k) {
      const int e = threadIdx.x + k * NT;
      float2 v;
      if (FROM_FX)
         v = grid_word((long long)stage[e], packed, inv);
      else
         v = reinterpret_cast<const float2*>(stage)[e];
      rowt[(e / N) * LDR + fsig<T>(e % N)] = v;
   }
   if (FROM_FX) {
      // the fixed-point slab is cleared for the next spread
      long long* q = qfx + base;
#pragma unroll
      for (int k = 0; k < PER; ++k)
         q[threadIdx.x + k * NT] = 0;
   }
   __syncthreads();
   const int line = threadIdx.x / T, t = threadIdx.x % T;
   float2 wt[N / T];
   fft_twiddles<N, T>(t, tw, wt);
   fft_line<N, T, INV>(rowt + line * LDR, 1, t, tw, wt);  // row rank R + line, along x
   // every CTA's rows transformed before any column gather
   asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
   // columns [rank R, rank R + R) of all N rows, from the owners' row tiles;
   // all PER remote loads are issued before any store
   const unsigned rowt_s = (unsigned)__cvta_generic_to_shared(rowt);
   float2 v[PER];
#pragma unroll
   for (int k = 0; k < PER; ++k) {
      const int e = threadIdx.x + k * NT;
      const int y = e / R, xl = e % R;
      const unsigned owner = (unsigned)(y / R);
      const unsigned local = rowt_s + (unsigned)(((y % R) * LDR + fsig<T>((int)rank * R + xl)) * sizeof(float2));
      unsigned remote;
      asm volatile("mapa.shared::cluster.u32 %0, %1, %2;" : "=r"(remote) : "r"(local), "r"(owner));
      // volatile keeps the loads after the cluster barrier; no memory clobber, so they pipeline
      asm volatile("ld.shared::cluster.v2.f32 {%0, %1}, [%2];" : "=f"(v[k].x), "=f"(v[k].y) : "r"(remote));
   }
#pragma unroll
   for (int k = 0; k < PER; ++k) {
      const int e = threadIdx.x + k * NT;
      colt[fsig<T>(e / R) * LDC + e % R] = v[k];
   }
   __syncthreads();
   fft_line<N, T, INV>(colt + line, LDC, t, tw, wt);  // column rank R + line, along y
   __syncthreads();
   float2* out = g + (size_t)z * N * N + (size_t)rank * R;
#pragma unroll
   for (int k = 0; k < PER; ++k) {
      const int e = threadIdx.x + k * NT;
      const int y = e / R, xl = e % R;
      out[(size_t)y * N + xl] = colt[fsig<T>(y) * LDC + xl];
   }
   // no CTA leaves while a peer may still read its row tile
   asm volatile("barrier.cluster.arrive.release.aligned;\nbarrier.cluster.wait.acquire.aligned;" ::: "memory");
}

template <int N, int CL, bool FROM_FX, bool INV>
static cudaError_t launch_plane_cl(long long* qfx, float2* g, int packed, float inv, int* err, cudaStream_t st)
{
   using C = PlaneCl<N, CL>;
   cudaLaunchConfig_t cfg = {};
   cfg.gridDim = dim3(N * CL);
   cfg.blockDim = dim3(C::NT);
   cfg.dynamicSmemBytes = C::SMEM;
   cfg.stream = st;
   cudaLaunchAttribute at[1];
   at[0].id = cudaLaunchAttributeClusterDimension;
   at[0].val.clusterDim.x = CL;
   at[0].val.clusterDim.y = 1;
   at[0].val.clusterDim.z = 1;
   cfg.attrs = at;
   cfg.numAttrs = 1;
   return cudaLaunchKernelEx(&cfg, k_fft_plane_cl<N, CL, FROM_FX, INV>, qfx, g, packed, inv, err);
}

template <int N, int CL>
static int plane_cl_setup(Context* ctx)
{
   const int bytes = (int)PlaneCl<N, CL>::SMEM;
   T9_CUDA(cudaFuncSetAttribute(k_fft_plane_cl<N, CL, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      bytes));
   T9_CUDA(cudaFuncSetAttribute(k_fft_plane_cl<N, CL, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
      bytes));
   return T9GB_OK;
}

template <int N>
static size_t fft_plane_smem()
{
   return sizeof(float2) * ((size_t)N * fft_plane_ld<N>() + 128);
}

// plane pass with clusters of P.fft_cl CTAs (0: one CTA per plane)
template <int N, bool FROM_FX, bool INV>
static void plane_pass(const PmeGrid& P, cudaStream_t st, int packed, float inv, bool pdl, int* range)
{
   constexpr int T = fft_threads_per_line<N>();
   if (P.fft_cl == 2)
      launch_plane_cl<N, 2, FROM_FX, INV>(P.qfx, P.qgrid, packed, inv, P.fft_err, st);
   else if (P.fft_cl == 4)
      launch_plane_cl<N, 4, FROM_FX, INV>(P.qfx, P.qgrid, packed, inv, P.fft_err, st);
   else if (P.fft_cl == 8)
      launch_plane_cl<N, 8, FROM_FX, INV>(P.qfx, P.qgrid, packed, inv, P.fft_err, st);
   else
      launch_k(pdl, k_fft_plane<N, FROM_FX, INV>, N, N * T, fft_plane_smem<N>(), st, P.qfx, P.qgrid, packed, inv,
         range);
}


template <int N>
static int fft_setup_kernels(Context* ctx)
{
   int rc = plane_cl_setup<N, 2>(ctx);
   if (rc == T9GB_OK)
      rc = plane_cl_setup<N, 4>(ctx);
   if (rc == T9GB_OK && N >= 64)
      rc = plane_cl_setup<N, 8>(ctx);
   T9_CHECK(rc);
   const int bytes = (int)fft_plane_smem<N>();
   void (*fwd)(long long*, float2*, int, float, int*) = k_fft_plane<N, true, false>;
   void (*inv)(long long*, float2*, int, float, int*) = k_fft_plane<N, false, true>;
   T9_CUDA(cudaFuncSetAttribute(fwd, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
   T9_CUDA(cudaFuncSetAttribute(inv, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes));
   return T9GB_OK;
}

// forward planes; vir: the z pass stops after the forward transform
template <int N>
static void fft_own_forward(const PmeGrid& P, cudaStream_t st, bool split, bool pdl, int* range)
{
   constexpr int T = fft_threads_per_line<N>();
   plane_pass<N, true, false>(P, st, P.packed ? 1 : 0, 1.0f / (float)(1 << P.pack_shift), pdl, range);
   if (split)
      launch_k(pdl, k_fft_zline<N, 0>, N * N / 16, 16 * T, 0, st, P.infl, P.qgrid);
   else
      launch_k(pdl, k_fft_zline<N, 2>, N * N / 16, 16 * T, 0, st, P.infl, P.qgrid);
}

template <int N>
static void fft_own_inverse(const PmeGrid& P, cudaStream_t st, bool split, bool pdl)
{
   constexpr int T = fft_threads_per_line<N>();
   if (split)
      launch_k(pdl, k_fft_zline<N, 1>, N * N / 16, 16 * T, 0, st, P.infl, P.qgrid);
   plane_pass<N, false, true>(P, st, 0, 0.f, pdl, nullptr);
}

// ---------------------------------------------------------------------------
// k-space part of the reciprocal virial (the strain derivative of the
// influence function), read-only on the forward-transformed grid:
//   W_ab += sum_m w(m) G(m) [-delta_ab + 2 h_a h_b (1 + pi^2 h^2 / a^2) / h^2]
// MODE 1 (permanent grid): w = wE |F(m)|^2, and the grid is kept in qstash
// when stash != null.  MODE 2 (d real, p imaginary): with
// Q_d = (F(m) + F*(-m)) / 2, Q_p = (F(m) - F*(-m)) / 2i and the kept
// permanent Q_M, w = wP Re[Q_M (Q_d + Q_p)* + Q_d Q_p*].  The reference's
// counterpart is pmeConv_cu1<Do_V> (src/cu/pme.cu:908-1031).  Six sums in a
// fixed order; the last block writes them to out[0..6) (xx yy zz xy xz yz).
template <int MODE>
__global__ void k_conv_virial(int n1, int n2, int n3, float L1, float L2, float L3, float pterm,
   const float* __restrict__ infl, const float2* __restrict__ g, float2* __restrict__ stash, float wE, float wP,
   double* __restrict__ red, double* __restrict__ out, int* __restrict__ state)
{
   __shared__ double sh[64];
   float v[6] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f};  // FP32 per thread and warp, FP64 above
   const size_t ng = (size_t)n1 * n2 * n3;
   for (size_t i = blockIdx.x * (size_t)blockDim.x + threadIdx.x; i < ng; i += (size_t)gridDim.x * blockDim.x) {
      const int k1 = (int)(i % n1), k2 = (int)((i / n1) % n2), k3 = (int)(i / ((size_t)n1 * n2));
      const float2 F = g[i];
      float2 QM = make_float2(0.f, 0.f);
      if (MODE == 1 && stash)
         stash[i] = F;
      if (MODE == 2)
         QM = stash[i];
      if (i == 0)
         continue;
      const int r1 = (k1 < (n1 + 1) / 2) ? k1 : k1 - n1;
      const int r2 = (k2 < (n2 + 1) / 2) ? k2 : k2 - n2;
      const int r3 = (k3 < (n3 + 1) / 2) ? k3 : k3 - n3;
      const float h[3] = {r1 / L1, r2 / L2, r3 / L3};
      const float hsq = h[0] * h[0] + h[1] * h[1] + h[2] * h[2];
      // per-point terms in FP32; the block and grid sums in FP64
      float w;
      if (MODE == 1) {
         w = wE * (F.x * F.x + F.y * F.y);
      } else {
         const int m1 = k1 == 0 ? 0 : n1 - k1, m2 = k2 == 0 ? 0 : n2 - k2, m3 = k3 == 0 ? 0 : n3 - k3;
         const float2 Fm = g[((size_t)m3 * n2 + m2) * n1 + m1];
         // Q_d = (F + conj(Fm)) / 2, Q_p = (F - conj(Fm)) / (2i)
         const float dx = 0.5f * (F.x + Fm.x), dy = 0.5f * (F.y - Fm.y);
         const float px = 0.5f * (F.y + Fm.y), py = -0.5f * (F.x - Fm.x);
         const float ux = dx + px, uy = dy + py;
         w = wP * ((QM.x * ux + QM.y * uy) + (dx * px + dy * py));
      }
      w *= infl[i];
      const float wf = w * (2.f * (1.f + pterm * hsq) / hsq);
      v[0] += wf * h[0] * h[0] - w;
      v[1] += wf * h[1] * h[1] - w;
      v[2] += wf * h[2] * h[2] - w;
      v[3] += wf * h[0] * h[1];
      v[4] += wf * h[0] * h[2];
      v[5] += wf * h[1] * h[2];
   }
   store_partials_f<6>(red, 0, v, sh);
   if (!last_block(state + ST_TICKET0))
      return;
   double t[4];
   sum_slots(red, 0, 4, gridDim.x, sh, t);
   double t2[4];
   sum_slots(red, 4, 2, gridDim.x, sh, t2);
   if (threadIdx.x == 0) {
      out[0] = t[0];
      out[1] = t[1];
      out[2] = t[2];
      out[3] = t[3];
      out[4] = t2[0];
      out[5] = t2[1];
   }
}

// ---------------------------------------------------------------------------
// Force gathers: the 20 fractional derivatives of the reciprocal potential
// (level-4 weights; the reference's fphi order: 0, x, y, z, xx, yy, zz, xy,
// xz, yz, xxx, yyy, zzz, xxy, xxz, xyy, yyz, xzz, yzz, xyz), made Cartesian
// (orthogonal box: one factor nfft/L per derivative) and contracted on the
// spot.  Replaces fphiMpole/fphiUind (src/cu/pme.cu:383-906) followed by the
// force/torque parts of empoleEwaldRecipGeneric_cu (src/cu/hippo/empole.cu)
// and epolarEwaldRecipSelf_cu1 (src/cu/epolarrecip.cu:414-511).

__device__ __forceinline__ void row_sums20(const float2* __restrict__ g, const GridParams& G, int i1, size_t row,
   const float (*t1)[4], bool imag, float* t)
{
   t[0] = t[1] = t[2] = t[3] = 0.f;
#pragma unroll
   for (int ix = 0; ix < 5; ++ix) {
      int xb = i1 + ix;
      xb -= (xb >= G.n1 ? G.n1 : 0);
      const float2 qv = g[row + xb];
      const float q = imag ? qv.y : qv.x;
#pragma unroll
      for (int l = 0; l < 4; ++l)
         t[l] += q * t1[ix][l];
   }
}

// row idx of a [5][L] weight table without dynamic indexing (keeps the
// table in registers)
template <int L>
__device__ __forceinline__ void pick_row(const float (*t)[L], int idx, float* out)
{
#pragma unroll
   for (int l = 0; l < L; ++l)
      out[l] = t[0][l];
#pragma unroll
   for (int j = 1; j < 5; ++j)
      if (idx == j)
#pragma unroll
         for (int l = 0; l < L; ++l)
            out[l] = t[j][l];
}

__device__ __forceinline__ void fphi20(const float* t, const float* u, const float* v, float* phi)
{
   phi[0] = t[0] * u[0] * v[0];
   phi[1] = t[1] * u[0] * v[0];
   phi[2] = t[0] * u[1] * v[0];
   phi[3] = t[0] * u[0] * v[1];
   phi[4] = t[2] * u[0] * v[0];
   phi[5] = t[0] * u[2] * v[0];
   phi[6] = t[0] * u[0] * v[2];
   phi[7] = t[1] * u[1] * v[0];
   phi[8] = t[1] * u[0] * v[1];
   phi[9] = t[0] * u[1] * v[1];
   phi[10] = t[3] * u[0] * v[0];
   phi[11] = t[0] * u[3] * v[0];
   phi[12] = t[0] * u[0] * v[3];
   phi[13] = t[2] * u[1] * v[0];
   phi[14] = t[2] * u[0] * v[1];
   phi[15] = t[1] * u[2] * v[0];
   phi[16] = t[0] * u[2] * v[1];
   phi[17] = t[1] * u[0] * v[2];
   phi[18] = t[0] * u[1] * v[2];
   phi[19] = t[1] * u[1] * v[1];
}

// fractional -> Cartesian for the 20 derivatives
__device__ __forceinline__ void to_cart20(const GridParams& G, float* c)
{
   const float a = G.a1, b = G.a2, d = G.a3;
   c[1] *= a;
   c[2] *= b;
   c[3] *= d;
   c[4] *= a * a;
   c[5] *= b * b;
   c[6] *= d * d;
   c[7] *= a * b;
   c[8] *= a * d;
   c[9] *= b * d;
   c[10] *= a * a * a;
   c[11] *= b * b * b;
   c[12] *= d * d * d;
   c[13] *= a * a * b;
   c[14] *= a * a * d;
   c[15] *= a * b * b;
   c[16] *= b * b * d;
   c[17] *= a * d * d;
   c[18] *= b * d * d;
   c[19] *= a * b * d;
}

__device__ __forceinline__ int ix2(int a, int b)
{
   return a == b ? 4 + a : (a + b == 1 ? 7 : (a + b == 2 ? 8 : 9));
}

__device__ __forceinline__ int ix3(int a, int b, int c)
{
   int n[3] = {0, 0, 0};
   n[a]++;
   n[b]++;
   n[c]++;
   if (n[0] == 3)
      return 10;
   if (n[1] == 3)
      return 11;
   if (n[2] == 3)
      return 12;
   if (n[0] == 2)
      return n[1] ? 13 : 14;
   if (n[1] == 2)
      return n[0] ? 15 : 16;
   if (n[2] == 2)
      return n[0] ? 17 : 18;
   return 19;
}

// -(q phi_a + d_b phi_ab + Theta_bc phi_abc) for a multipole row m (12 floats)
__device__ __forceinline__ void mpole_force(const float* m, const float* c, float* F)
{
   const float Q[3][3] = {{m[4], m[7], m[8]}, {m[7], m[5], m[9]}, {m[8], m[9], m[6]}};
#pragma unroll
   for (int a = 0; a < 3; ++a) {
      float v = m[0] * c[1 + a];
#pragma unroll
      for (int b = 0; b < 3; ++b) {
         v += m[1 + b] * c[ix2(a, b)];
#pragma unroll
         for (int cc = 0; cc < 3; ++cc)
            v += Q[b][cc] * c[ix3(a, b, cc)];
      }
      F[a] = -v;
   }
}

// permanent grid: multipole forces, torque field and energies (MPOLE), the
// polarization force on the dipoles in the permanent field gradient and the
// Ewald self torque (POLAR)
// wout (may be null): the fractional-transform part of the virial per slot,
// [9][npad]; the dipole-grid gather adds to the same rows
template <bool MPOLE, bool POLAR>
__global__ void __launch_bounds__(256) k_gather_force_perm(int n, int npad, GridParams G, float f, float aewald,
   const float4* __restrict__ spos, const float2* __restrict__ g, const float* __restrict__ rp,
   const float* __restrict__ u8, float* __restrict__ fout, float* __restrict__ tout, double* __restrict__ e_atom,
   double* __restrict__ e_self, float* __restrict__ wout)
{
   const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int lane = threadIdx.x & 31;
   if (s >= n)
      return;
   int i1, i2, i3;
   float w1, w2, w3;
   site(G, spos[s], i1, i2, i3, w1, w2, w3);
   float phi[20];
#pragma unroll
   for (int c = 0; c < 20; ++c)
      phi[c] = 0.f;
   if (lane < 25) {
      float t1[5][4], t2[5][4], t3[5][4];
      bspline5<4>(w1, t1);
      bspline5<4>(w2, t2);
      bspline5<4>(w3, t3);
      const int jy = lane % 5, kz = lane / 5;
      int zb = i3 + kz;
      zb -= (zb >= G.n3 ? G.n3 : 0);
      int yb = i2 + jy;
      yb -= (yb >= G.n2 ? G.n2 : 0);
      const size_t row = ((size_t)zb * G.n2 + yb) * G.n1;
      float t[4], uy[4], vz[4];
      pick_row<4>(t2, jy, uy);
      pick_row<4>(t3, kz, vz);
      row_sums20(g, G, i1, row, t1, false, t);
      fphi20(t, uy, vz, phi);
   }
#pragma unroll
   for (int c = 0; c < 20; ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         phi[c] += __shfl_xor_sync(0xffffffffu, phi[c], o);
   if (lane != 0)
      return;
   to_cart20(G, phi);
   const float* m = rp + 12 * s;
   float F[3] = {0.f, 0.f, 0.f}, T[10];
#pragma unroll
   for (int c = 0; c < 10; ++c)
      T[c] = 0.f;
   if (MPOLE) {
      mpole_force(m, phi, F);
      #pragma unroll
      for (int c = 0; c < 3; ++c)
         F[c] *= f;
      #pragma unroll
      for (int c = 0; c < 10; ++c)
         T[c] = f * phi[c];
      // per-atom energies in FP32 (this GPU's FP64 pipe issues a warp
      // instruction in tens of cycles even for one lane); the totals are
      // FP64 sums of these
      if (e_atom) {
         float e = m[0] * phi[0] + m[1] * phi[1] + m[2] * phi[2] + m[3] * phi[3];
         e += m[4] * phi[4] + m[5] * phi[5] + m[6] * phi[6];
         e += 2.f * (m[7] * phi[7] + m[8] * phi[8] + m[9] * phi[9]);
         e_atom[s] = (double)(0.5f * f * e);
      }
      if (e_self) {
         const float a2 = 2.f * aewald * aewald;
         const float fterm = -f * aewald * 0.56418958354775628f;  // 1/sqrt(pi)
         const float cii = m[0] * m[0];
         const float dii = m[1] * m[1] + m[2] * m[2] + m[3] * m[3];
         const float qii = 2.f * (m[7] * m[7] + m[8] * m[8] + m[9] * m[9]) + m[4] * m[4] + m[5] * m[5] + m[6] * m[6];
         e_self[s] = (double)(fterm * (cii + a2 * (dii * (1.f / 3.f) + 0.4f * a2 * qii)));
      }
   }
   float us[3] = {0.f, 0.f, 0.f};
   if (POLAR) {
      const float* u = u8 + 8 * s;
      us[0] = u[0] + u[3];
      us[1] = u[1] + u[4];
      us[2] = u[2] + u[5];
#pragma unroll
      for (int a = 0; a < 3; ++a) {
         float v = 0.f;
#pragma unroll
         for (int b = 0; b < 3; ++b)
            v += us[b] * phi[ix2(a, b)];
         F[a] -= 0.5f * f * v;
         T[1 + a] -= 0.5f * f * G.selfterm * us[a];
      }
   }
   #pragma unroll
   for (int c = 0; c < 3; ++c)
      fout[3 * s + c] = F[c];
   #pragma unroll
   for (int c = 0; c < 10; ++c)
      tout[10 * s + c] = T[c];
   if (wout) {
      // -f [phi_a d_b + 2 (phi2 Theta)_ab] (MPOLE), -f/2 phi_a u_b (POLAR)
      const float Q[3][3] = {{m[4], m[7], m[8]}, {m[7], m[5], m[9]}, {m[8], m[9], m[6]}};
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
         for (int b = 0; b < 3; ++b) {
            float w = 0.f;
            if (MPOLE) {
               float pq = 0.f;
#pragma unroll
               for (int c = 0; c < 3; ++c)
                  pq += phi[ix2(a, c)] * Q[c][b];
               w -= f * (phi[1 + a] * m[1 + b] + 2.f * pq);
            }
            if (POLAR)
               w -= 0.5f * f * phi[1 + a] * us[b];
            wout[(3 * a + b) * npad + s] = w;
         }
   }
}

// induced-dipole grid (d real, p imaginary): force on the multipoles in the
// dipoles' potential, the mutual dipole force and the torque field
__global__ void __launch_bounds__(256) k_gather_force_uind(int n, int npad, GridParams G, float f,
   const float4* __restrict__ spos, const float2* __restrict__ g, const float* __restrict__ rp,
   const float* __restrict__ u8, float* __restrict__ fout, float* __restrict__ tout, float* __restrict__ wout)
{
   const int s = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int lane = threadIdx.x & 31;
   if (s >= n)
      return;
   int i1, i2, i3;
   float w1, w2, w3;
   site(G, spos[s], i1, i2, i3, w1, w2, w3);
   float pd[20], pp[20];
#pragma unroll
   for (int c = 0; c < 20; ++c)
      pd[c] = pp[c] = 0.f;
   if (lane < 25) {
      float t1[5][4], t2[5][4], t3[5][4];
      bspline5<4>(w1, t1);
      bspline5<4>(w2, t2);
      bspline5<4>(w3, t3);
      const int jy = lane % 5, kz = lane / 5;
      int zb = i3 + kz;
      zb -= (zb >= G.n3 ? G.n3 : 0);
      int yb = i2 + jy;
      yb -= (yb >= G.n2 ? G.n2 : 0);
      const size_t row = ((size_t)zb * G.n2 + yb) * G.n1;
      float t[4], uy[4], vz[4];
      pick_row<4>(t2, jy, uy);
      pick_row<4>(t3, kz, vz);
      row_sums20(g, G, i1, row, t1, false, t);
      fphi20(t, uy, vz, pd);
      row_sums20(g, G, i1, row, t1, true, t);
      fphi20(t, uy, vz, pp);
   }
#pragma unroll
   for (int c = 0; c < 20; ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
         pd[c] += __shfl_xor_sync(0xffffffffu, pd[c], o);
         pp[c] += __shfl_xor_sync(0xffffffffu, pp[c], o);
      }
   if (lane != 0)
      return;
   to_cart20(G, pd);
   to_cart20(G, pp);
   float ps[20];
   #pragma unroll
   for (int c = 0; c < 20; ++c)
      ps[c] = pd[c] + pp[c];
   const float* m = rp + 12 * s;
   const float* u = u8 + 8 * s;
   float F[3];
   mpole_force(m, ps, F);
#pragma unroll
   for (int a = 0; a < 3; ++a) {
      float v = 0.f;
#pragma unroll
      for (int b = 0; b < 3; ++b)
         v += u[b] * pp[ix2(a, b)] + u[3 + b] * pd[ix2(a, b)];
      fout[3 * s + a] = 0.5f * f * (F[a] - v);
   }
   #pragma unroll
   for (int c = 0; c < 10; ++c)
      tout[10 * s + c] = 0.5f * f * ps[c];
   if (wout) {
      // -f/2 [psi_a d_b + 2 (psi2 Theta)_ab + psi^p_a u_d,b + psi^d_a u_p,b]
      const float Q[3][3] = {{m[4], m[7], m[8]}, {m[7], m[5], m[9]}, {m[8], m[9], m[6]}};
#pragma unroll
      for (int a = 0; a < 3; ++a)
#pragma unroll
         for (int b = 0; b < 3; ++b) {
            float pq = 0.f;
#pragma unroll
            for (int c = 0; c < 3; ++c)
               pq += ps[ix2(a, c)] * Q[c][b];
            const float w = ps[1 + a] * m[1 + b] + 2.f * pq + pp[1 + a] * u[b] + pd[1 + a] * u[3 + b];
            wout[(3 * a + b) * npad + s] -= 0.5f * f * w;
         }
   }
}

// ---------------------------------------------------------------------------

int pme_setup(Context* ctx)
{
   const t9gb_config& c = ctx->cfg;
   PmeGrid& P = ctx->pme;
   if (!c.use_ewald)
      return T9GB_OK;
   P.n1 = c.nfft[0];
   P.n2 = c.nfft[1];
   P.n3 = c.nfft[2];
   const size_t ng = (size_t)P.n1 * P.n2 * P.n3;
   T9_CUDA(cudaMalloc(&P.qgrid, sizeof(float2) * ng));
   T9_CUDA(cudaMalloc(&P.qfx, sizeof(long long) * ng));
   T9_CUDA(cudaMemset(P.qfx, 0, sizeof(long long) * ng));
   // the second grid: the induced-dipole half of the reciprocal forces runs
   // beside the permanent half
   T9_CUDA(cudaMalloc(&P.qgrid2, sizeof(float2) * ng));
   T9_CUDA(cudaMalloc(&P.qfx2, sizeof(long long) * ng));
   T9_CUDA(cudaMemset(P.qfx2, 0, sizeof(long long) * ng));
   // influence function in double precision, stored as float
   std::vector<double> m1, m2, m3;
   bspline_moduli(P.n1, c.bsorder, m1);
   bspline_moduli(P.n2, c.bsorder, m2);
   bspline_moduli(P.n3, c.bsorder, m3);
   const double pi = 3.14159265358979323846;
   const double pterm = (pi / c.aewald) * (pi / c.aewald);
   const double vol = c.box[0] * c.box[1] * c.box[2];
   std::vector<float> infl(ng);
   for (int k3 = 0; k3 < P.n3; ++k3)
      for (int k2 = 0; k2 < P.n2; ++k2)
         for (int k1 = 0; k1 < P.n1; ++k1) {
            size_t i = ((size_t)k3 * P.n2 + k2) * P.n1 + k1;
            int r1 = (k1 < (P.n1 + 1) / 2) ? k1 : k1 - P.n1;
            int r2 = (k2 < (P.n2 + 1) / 2) ? k2 : k2 - P.n2;
            int r3 = (k3 < (P.n3 + 1) / 2) ? k3 : k3 - P.n3;
            double h1 = r1 / c.box[0], h2 = r2 / c.box[1], h3 = r3 / c.box[2];
            double hsq = h1 * h1 + h2 * h2 + h3 * h3;
            double term = -pterm * hsq;
            double e = 0;
            if (i != 0 && term > -50)
               e = std::exp(term) / (hsq * pi * vol * m1[k1] * m2[k2] * m3[k3]);
            infl[i] = (float)e;
         }
   float* d_infl = nullptr;
   T9_CUDA(cudaMalloc(&d_infl, sizeof(float) * ng));
   T9_CUDA(cudaMemcpy(d_infl, infl.data(), sizeof(float) * ng, cudaMemcpyHostToDevice));
   P.infl = d_infl;
   T9_CUDA(cudaMalloc(&P.fft_err, sizeof(int)));
   T9_CUDA(cudaMemset(P.fft_err, 0, sizeof(int)));
   if (cufftPlan3d(&P.plan, P.n3, P.n2, P.n1, CUFFT_C2C) != CUFFT_SUCCESS ||
      cufftPlan3d(&P.plan2, P.n3, P.n2, P.n1, CUFFT_C2C) != CUFFT_SUCCESS) {
      ctx->last_error = "cufftPlan3d failed";
      return T9GB_CUDA_ERR;
   }
   // the fused FFT: cubic grids of 32, 64 or 128 points per edge
   P.own_fft_ok = P.n1 == P.n2 && P.n2 == P.n3 && (P.n1 == 32 || P.n1 == 64 || P.n1 == 128);
   // default where it measured faster than cuFFT on GB300 (64^3: 0.627 vs
   // 0.634 ms per induce step in the graph); at 128^3 cuFFT is faster
   P.own_fft = P.own_fft_ok && P.n1 <= 64;
   if (P.own_fft_ok) {
      if (P.n1 == 32)
         T9_CHECK(fft_setup_kernels<32>(ctx));
      else if (P.n1 == 64)
         T9_CHECK(fft_setup_kernels<64>(ctx));
      else
         T9_CHECK(fft_setup_kernels<128>(ctx));
      float2 tw[128];
      for (int k = 0; k < 128; ++k)
         tw[k] = make_float2((float)std::cos(2 * pi * k / 128.0), (float)-std::sin(2 * pi * k / 128.0));
      T9_CUDA(cudaMemcpyToSymbol(c_tw, tw, sizeof(tw)));
      T9_CUDA(cudaDeviceSynchronize());
   }
   return T9GB_OK;
}

void pme_free(Context* ctx)
{
   PmeGrid& P = ctx->pme;
   if (P.plan)
      cufftDestroy(P.plan);
   if (P.plan2)
      cufftDestroy(P.plan2);
   cudaFree(P.qgrid2);
   cudaFree(P.qfx2);
   cudaFree(P.qgrid);
   cudaFree(P.qfx);
   cudaFree(P.infl);
   cudaFree(P.qstash);
   cudaFree(P.fft_err);
   P = PmeGrid();
}

static GridParams grid_params(const Context* ctx)
{
   const t9gb_config& c = ctx->cfg;
   GridParams G;
   G.n1 = c.nfft[0];
   G.n2 = c.nfft[1];
   G.n3 = c.nfft[2];
   G.r1 = (float)(1.0 / c.box[0]);
   G.r2 = (float)(1.0 / c.box[1]);
   G.r3 = (float)(1.0 / c.box[2]);
   G.a1 = (float)(c.nfft[0] / c.box[0]);
   G.a2 = (float)(c.nfft[1] / c.box[1]);
   G.a3 = (float)(c.nfft[2] / c.box[2]);
   G.selfterm = (float)(4.0 * c.aewald * c.aewald * c.aewald / (3.0 * 1.77245385090551602730));
   G.pk_s = (float)(1 << ctx->pme.pack_shift);
   G.pk_lim = (float)(1 << (31 - 5 - ctx->pme.pack_shift));
   G.range = ctx->status + (ctx->pme.probe ? ST_RANGE_L : ST_RANGE);
   return G;
}

static int conv_virial(Context* ctx, int vir, float wE, float wP, bool stash, double* out)
{
   PmeGrid& P = ctx->pme;
   const size_t ng = (size_t)P.n1 * P.n2 * P.n3;
   const t9gb_config& c = ctx->cfg;
   const float pterm = (float)((3.14159265358979323846 / c.aewald) * (3.14159265358979323846 / c.aewald));
   if ((stash || vir == 2) && !P.qstash)
      T9_CUDA(cudaMalloc(&P.qstash, sizeof(float2) * ng));
   const int vb = (int)std::min<size_t>((ng + 255) / 256, RED_MAX);
   if (vir == 1)
      k_conv_virial<1><<<vb, 256, 0, ctx->stream>>>(P.n1, P.n2, P.n3, (float)c.box[0], (float)c.box[1],
         (float)c.box[2], pterm, P.infl, P.qgrid, stash ? P.qstash : nullptr, wE, wP, ctx->red, out, ctx->status);
   else
      k_conv_virial<2><<<vb, 256, 0, ctx->stream>>>(P.n1, P.n2, P.n3, (float)c.box[0], (float)c.box[1],
         (float)c.box[2], pterm, P.infl, P.qgrid, P.qstash, wE, wP, ctx->red, out, ctx->status);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// vir: 0 none, 1 permanent-grid k-space virial (wE, stash), 2 dipole-grid
// cross terms (wP); the sums go to out[0..6)
static int fft_conv(Context* ctx, int vir = 0, float wE = 0.f, float wP = 0.f, bool stash = false,
   double* out = nullptr)
{
   PmeGrid& P = ctx->pme;
   const size_t ng = (size_t)P.n1 * P.n2 * P.n3;
   const int cb = (int)std::min<size_t>((ng + 255) / 256, 152 * 16);
   prof_begin(ctx, P_FFT_CONV);
   int* range = ctx->status + (P.probe ? ST_RANGE_L : ST_RANGE);
   if (P.own_fft) {
      cudaStream_t st = ctx->stream;
      const bool split = vir != 0;
      const bool pdl = use_pdl(ctx);
      if (P.n1 == 32)
         fft_own_forward<32>(P, st, split, pdl, range);
      else if (P.n1 == 64)
         fft_own_forward<64>(P, st, split, pdl, range);
      else
         fft_own_forward<128>(P, st, split, pdl, range);
      if (split) {
         T9_CHECK(conv_virial(ctx, vir, wE, wP, stash, out));
         k_conv<<<cb, 256, 0, st>>>(ng, P.infl, P.qgrid);
      }
      if (P.n1 == 32)
         fft_own_inverse<32>(P, st, split, pdl && !split);
      else if (P.n1 == 64)
         fft_own_inverse<64>(P, st, split, pdl && !split);
      else
         fft_own_inverse<128>(P, st, split, pdl && !split);
      T9_CUDA(cudaGetLastError());
      prof_end(ctx);
      return T9GB_OK;
   }
   k_fx_to_grid<<<cb, 256, 0, ctx->stream>>>(ng, P.qfx, P.qgrid, P.packed ? 1 : 0,
      1.0f / (float)(1 << P.pack_shift), range);
   T9_CUDA(cudaGetLastError());
   cufftSetStream(P.plan, ctx->stream);
   if (cufftExecC2C(P.plan, (cufftComplex*)P.qgrid, (cufftComplex*)P.qgrid, CUFFT_FORWARD) != CUFFT_SUCCESS) {
      ctx->last_error = "cufftExecC2C forward failed";
      return T9GB_CUDA_ERR;
   }
   if (vir)
      T9_CHECK(conv_virial(ctx, vir, wE, wP, stash, out));
   k_conv<<<cb, 256, 0, ctx->stream>>>(ng, P.infl, P.qgrid);
   T9_CUDA(cudaGetLastError());
   if (cufftExecC2C(P.plan, (cufftComplex*)P.qgrid, (cufftComplex*)P.qgrid, CUFFT_INVERSE) != CUFFT_SUCCESS) {
      ctx->last_error = "cufftExecC2C inverse failed";
      return T9GB_CUDA_ERR;
   }
   prof_end(ctx);
   return T9GB_OK;
}

// Reciprocal permanent field in two halves: the grid (spread + transform,
// on ctx->stream) and the gather (recip + self into out6; acc: added to the
// real-space field stored there)
int launch_dfield_recip_grid(Context* ctx)
{
   if (!ctx->cfg.use_ewald)
      return T9GB_OK;
   GridParams G = grid_params(ctx);
   prof_begin(ctx, P_SPREAD_MPOLE);
   ctx->pme.packed = false;
   k_spread<0><<<grid_for((long long)ctx->n * 32, 256), 256, 0, ctx->stream>>>(ctx->n, G, ctx->spos, ctx->srpole,
      nullptr, nullptr, reinterpret_cast<unsigned long long*>(ctx->pme.qfx));
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return fft_conv(ctx);
}

int launch_dfield_recip_gather(Context* ctx, float* out6, bool acc)
{
   if (!ctx->cfg.use_ewald)
      return T9GB_OK;
   GridParams G = grid_params(ctx);
   const int nb = grid_for((long long)ctx->n * 32, 256);
   prof_begin(ctx, P_GATHER_MPOLE);
   if (acc)
      k_gather_field<0, true><<<nb, 256, 0, ctx->stream>>>(ctx->n, G, ctx->spos, ctx->pme.qgrid, ctx->srpole, nullptr,
         out6, PcgAp{});
   else
      k_gather_field<0, false><<<nb, 256, 0, ctx->stream>>>(ctx->n, G, ctx->spos, ctx->pme.qgrid, ctx->srpole,
         nullptr, out6, PcgAp{});
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int launch_dfield_recip(Context* ctx, float* out6)
{
   T9_CHECK(launch_dfield_recip_grid(ctx));
   return launch_dfield_recip_gather(ctx, out6, false);
}

int launch_ufield_recip_grid(Context* ctx, const float* u6)
{
   if (!ctx->cfg.use_ewald)
      return T9GB_OK;
   GridParams G = grid_params(ctx);
   prof_begin(ctx, P_SPREAD_UIND);
   ctx->pme.packed = true;
   T9_CUDA(launch_k(use_pdl(ctx), k_spread<1, false>, grid_for((long long)ctx->n * 32, 256), 256, 0, ctx->stream,
      ctx->n, G, ctx->spos, u6, nullptr, nullptr, reinterpret_cast<unsigned long long*>(ctx->pme.qfx)));
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return fft_conv(ctx);
}

int launch_ufield_recip_gather(Context* ctx, const float* u6, float* out6, bool acc)
{
   if (!ctx->cfg.use_ewald)
      return T9GB_OK;
   GridParams G = grid_params(ctx);
   const int nb = grid_for((long long)ctx->n * 32, 256);
   prof_begin(ctx, P_GATHER_UIND);
   T9_CUDA(launch_k(use_pdl(ctx), acc ? k_gather_field<1, true> : k_gather_field<1, false>, nb, 256, 0, ctx->stream,
      ctx->n, G, ctx->spos, ctx->pme.qgrid, nullptr, u6, out6, PcgAp{}));
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int launch_ufield_recip(Context* ctx, const float* u6, float* out6)
{
   T9_CHECK(launch_ufield_recip_grid(ctx, u6));
   return launch_ufield_recip_gather(ctx, u6, out6, false);
}

static void swap_grids(PmeGrid& P)
{
   std::swap(P.qfx, P.qfx2);
   std::swap(P.qgrid, P.qgrid2);
   std::swap(P.plan, P.plan2);
}

int launch_ufield_recip_grid_alt(Context* ctx, const float* u6)
{
   swap_grids(ctx->pme);
   const int rc = launch_ufield_recip_grid(ctx, u6);
   swap_grids(ctx->pme);
   return rc;
}

int launch_ufield_recip_gather_alt(Context* ctx, const float* u6, float* out6)
{
   swap_grids(ctx->pme);
   const int rc = launch_ufield_recip_gather(ctx, u6, out6, true);
   swap_grids(ctx->pme);
   return rc;
}

// the CG search direction's grid: p = z + b p_old formed by the spread
int launch_ufield_recip_grid_dir(Context* ctx, const float* p6, const float* z6, const double* scal)
{
   if (!ctx->cfg.use_ewald)
      return T9GB_OK;
   GridParams G = grid_params(ctx);
   prof_begin(ctx, P_SPREAD_UIND);
   ctx->pme.packed = true;
   T9_CUDA(launch_k(use_pdl(ctx), k_spread<1, true>, grid_for((long long)ctx->n * 32, 256), 256, 0, ctx->stream,
      ctx->n, G, ctx->spos, p6, z6, scal, reinterpret_cast<unsigned long long*>(ctx->pme.qfx)));
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return fft_conv(ctx);
}

// recip + self field of the search direction p = z + b p_old (P.conj =
// p_old, P.zrsd = z, P.scal = b) added to the real-space field in out6
int launch_ufield_recip_gather_dir(Context* ctx, float* out6, const PcgAp& P)
{
   GridParams G = grid_params(ctx);
   const int nb = grid_for((long long)ctx->n * 32, 256);
   prof_begin(ctx, P_GATHER_UIND);
   k_gather_field<1, true, false, true><<<nb, 256, 0, ctx->stream>>>(ctx->n, G, ctx->spos, ctx->pme.qgrid, nullptr,
      nullptr, out6, P);
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// recip + self field of the search direction added to the real-space field
// in out6, then p, Ap and the step length (PcgAp)
int launch_ufield_recip_gather_ap(Context* ctx, float* out6, const PcgAp& P)
{
   GridParams G = grid_params(ctx);
   const int nb = std::min(RED_MAX, grid_for((long long)ctx->n * 32, 256));
   prof_begin(ctx, P_GATHER_UIND);
   k_gather_field<1, true, true><<<nb, 256, 0, ctx->stream>>>(ctx->n, G, ctx->spos, ctx->pme.qgrid, nullptr, nullptr,
      out6, P);
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

}  // namespace t9gb

namespace t9gb {
int launch_empole_recip(Context* ctx, double* e_atom)
{
   if (!ctx->cfg.use_ewald)
      return T9GB_OK;
   GridParams G = grid_params(ctx);
   ctx->pme.packed = false;
   k_spread<0><<<grid_for((long long)ctx->n * 32, 256), 256, 0, ctx->stream>>>(ctx->n, G, ctx->spos, ctx->srpole,
      nullptr, nullptr, reinterpret_cast<unsigned long long*>(ctx->pme.qfx));
   T9_CUDA(cudaGetLastError());
   T9_CHECK(fft_conv(ctx));
   k_empole_recip_self<<<grid_for((long long)ctx->n * 32, 256), 256, 0, ctx->stream>>>(ctx->n, G,
      (float)ctx->cfg.electric, (float)ctx->cfg.aewald, ctx->spos, ctx->pme.qgrid, ctx->srpole, e_atom,
      e_atom + ctx->npad);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}
}  // namespace t9gb

namespace t9gb {
// reciprocal forces for elec_forces (force.cu), in two halves: the
// permanent-multipole grid (forces and torque fields of the multipoles, the
// induced dipoles' force in the permanent field) and the induced-dipole
// grid.  wrec (may be null): the per-slot fractional-transform virial rows,
// k-space sums in scal[40..52); with the virial the dipole half reads the
// permanent half's transformed grid, so the two run in order.
int launch_force_recip_perm(Context* ctx, bool mpole, bool polar, float* wrec)
{
   GridParams G = grid_params(ctx);
   const int nb = grid_for((long long)ctx->n * 32, 256);
   const int np = ctx->npad;
   const float f = (float)ctx->cfg.electric, a = (float)ctx->cfg.aewald;
   const bool vir = wrec != nullptr;
   if (vir) {
      T9_CUDA(cudaMemsetAsync(wrec, 0, sizeof(float) * 9 * np, ctx->stream));
      T9_CUDA(cudaMemsetAsync(ctx->scal + 40, 0, sizeof(double) * 12, ctx->stream));
   }
   ctx->pme.packed = false;
   k_spread<0><<<nb, 256, 0, ctx->stream>>>(ctx->n, G, ctx->spos, ctx->srpole,
      nullptr, nullptr, reinterpret_cast<unsigned long long*>(ctx->pme.qfx));
   T9_CUDA(cudaGetLastError());
   T9_CHECK(fft_conv(ctx, vir ? 1 : 0, mpole ? 0.5f * f : 0.f, 0.f, vir && polar, ctx->scal + 40));
   double* er = ctx->e_atom + np;
   double* es = ctx->e_atom + 2 * np;
   if (mpole && polar)
      k_gather_force_perm<true, true><<<nb, 256, 0, ctx->stream>>>(ctx->n, np, G, f, a, ctx->spos, ctx->pme.qgrid,
         ctx->srpole, ctx->uind, ctx->frecp, ctx->trecp, er, es, wrec);
   else if (mpole)
      k_gather_force_perm<true, false><<<nb, 256, 0, ctx->stream>>>(ctx->n, np, G, f, a, ctx->spos, ctx->pme.qgrid,
         ctx->srpole, ctx->uind, ctx->frecp, ctx->trecp, er, es, wrec);
   else
      k_gather_force_perm<false, true><<<nb, 256, 0, ctx->stream>>>(ctx->n, np, G, f, a, ctx->spos, ctx->pme.qgrid,
         ctx->srpole, ctx->uind, ctx->frecp, ctx->trecp, nullptr, nullptr, wrec);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// alt: on the second grid (and FFT plan), so that it can run beside the
// permanent half on another stream (no virial)
int launch_force_recip_uind(Context* ctx, float* wrec, bool alt)
{
   PmeGrid& P = ctx->pme;
   if (alt) {
      std::swap(P.qfx, P.qfx2);
      std::swap(P.qgrid, P.qgrid2);
      std::swap(P.plan, P.plan2);
   }
   GridParams G = grid_params(ctx);
   const int nb = grid_for((long long)ctx->n * 32, 256);
   const float f = (float)ctx->cfg.electric;
   const bool vir = wrec != nullptr;
   P.packed = true;
   k_spread<1><<<nb, 256, 0, ctx->stream>>>(ctx->n, G, ctx->spos, ctx->uind,
      nullptr, nullptr, reinterpret_cast<unsigned long long*>(P.qfx));
   int rc = cudaGetLastError() == cudaSuccess ? T9GB_OK : T9GB_CUDA_ERR;
   if (rc == T9GB_OK)
      rc = fft_conv(ctx, vir ? 2 : 0, 0.f, 0.5f * f, false, ctx->scal + 46);
   if (rc == T9GB_OK) {
      k_gather_force_uind<<<nb, 256, 0, ctx->stream>>>(ctx->n, ctx->npad, G, f, ctx->spos, P.qgrid, ctx->srpole,
         ctx->uind, ctx->frecu, ctx->trecu, wrec);
      if (cudaGetLastError() != cudaSuccess)
         rc = T9GB_CUDA_ERR;
   }
   if (alt) {
      std::swap(P.qfx, P.qfx2);
      std::swap(P.qgrid, P.qgrid2);
      std::swap(P.plan, P.plan2);
   }
   return rc;
}

int launch_force_recip(Context* ctx, bool mpole, bool polar, float* wrec)
{
   T9_CHECK(launch_force_recip_perm(ctx, mpole, polar, wrec));
   if (polar)
      T9_CHECK(launch_force_recip_uind(ctx, wrec, false));
   return T9GB_OK;
}
}  // namespace t9gb
