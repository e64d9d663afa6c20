// Shared pieces of the real-space pair kernels (pair.cu, force.cu): pair
// parameters, minimum-image separation, fixed xor-tree group reductions and
// the 32-byte row load.
#pragma once
#include "common.cuh"

namespace t9gb {

struct PairParams {
   int n;
   float lx, ly, lz;     // box lengths (0 without PBC)
   float ilx, ily, ilz;  // inverse lengths (0 without PBC)
   float cut2;
   int ewald;
   float aewald;
   float ec1, ec2, ec3, ec4;  // (2a^2)^j / (sqrt(pi) a), j = 1..4
   int cap;              // list row stride
   const float* thl;     // per-type-pair Thole table [nthl][nthl], or null
   int nthl;
};

__device__ __forceinline__ float3 sep(const PairParams& P, float4 pi, float4 pk)
{
   return make_float3(image1(pk.x - pi.x, P.lx, P.ilx), image1(pk.y - pi.y, P.ly, P.ily),
      image1(pk.z - pi.z, P.lz, P.ilz));
}

// Thole coefficient of a pair from the two rows' thole slots: the
// per-type-pair table thlval[jpolar_i][jpolar_k] when one is set (the
// reference's CUDA pair kernels, src/cu/amoeba/ufield_cu1.cc, dfield_cu1.cc,
// sparsePrecond_cu1.cc, epolar_cu1.cc), else min(thole_i, thole_k)
// (damp_thole2/3, include/seq/damp.h:19-44)
__device__ __forceinline__ float pair_gamma(const PairParams& P, float ti, float tk)
{
   return P.thl ? __ldg(P.thl + (int)ti * P.nthl + (int)tk) : fminf(ti, tk);
}

template <int G, int N>
__device__ __forceinline__ void group_reduce(float* v)
{
#pragma unroll
   for (int c = 0; c < N; ++c) {
#pragma unroll
      for (int o = G / 2; o > 0; o >>= 1)
         v[c] += __shfl_xor_sync(0xffffffffu, v[c], o);
   }
}

// one 32-byte row: d xyz, p xyz, thole, polarizability
__device__ __forceinline__ void load8(const float* __restrict__ a, int s, float* v)
{
   const float4* p = reinterpret_cast<const float4*>(a + 8 * s);
   const float4 x = p[0], y = p[1];
   v[0] = x.x;
   v[1] = x.y;
   v[2] = x.z;
   v[3] = x.w;
   v[4] = y.x;
   v[5] = y.y;
   v[6] = y.z;
   v[7] = y.w;
}

static inline PairParams make_params(const Context* ctx, double cutoff)
{
   PairParams P;
   const t9gb_config& c = ctx->cfg;
   const bool pbc = c.box[0] > 0 && c.box[1] > 0 && c.box[2] > 0;
   P.n = ctx->n;
   P.lx = pbc ? (float)c.box[0] : 0.f;
   P.ly = pbc ? (float)c.box[1] : 0.f;
   P.lz = pbc ? (float)c.box[2] : 0.f;
   P.ilx = pbc ? (float)(1.0 / c.box[0]) : 0.f;
   P.ily = pbc ? (float)(1.0 / c.box[1]) : 0.f;
   P.ilz = pbc ? (float)(1.0 / c.box[2]) : 0.f;
   double cut2 = cutoff * cutoff;
   P.cut2 = cut2 > 3.0e38 ? 3.0e38f : (float)cut2;
   P.ewald = c.use_ewald;
   P.aewald = (float)c.aewald;
   const double a = c.aewald;
   const double alsq2 = 2 * a * a;
   const double base = a > 0 ? 1.0 / (1.77245385090551602730 * a) : 0.0;
   P.ec1 = (float)(base * alsq2);
   P.ec2 = (float)(base * alsq2 * alsq2);
   P.ec3 = (float)(base * alsq2 * alsq2 * alsq2);
   P.ec4 = (float)(base * alsq2 * alsq2 * alsq2 * alsq2);
   P.cap = ctx->nbr_cap;
   P.thl = ctx->nthl > 0 ? ctx->thl : nullptr;
   P.nthl = ctx->nthl;
   return P;
}

}  // namespace t9gb
