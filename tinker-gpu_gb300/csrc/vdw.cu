// Buffered 14-7 (HAL) van der Waals on the GPU: energy, gradient, virial.
//
// Restates the reference's ehal path (src/ehal.cpp, src/cu/ehal.cu,
// include/seq/pair_hal.h:52-96, switchTaper5 in include/math/switch.h:22-33):
//   E = eps (1.07 / (rho + 0.07))^7 (1.12 / (rho^7 + 0.12) - 2),  rho = r / R0,
// with R0 and eps from per-type-pair tables, the fifth-order taper between
// the taper and cutoff distances, scaled pairs (vdw-1x-scale) and reduced
// sites: an atom with a reduction factor red sits at x_p + red (x - x_p) of
// its parent p, and its site force goes back red to the atom and 1 - red to
// the parent.  The kernel walks the stored neighbour list (whose radius
// covers the cutoff plus the site margin) from both sides, so per-site sums
// are in a fixed order without atomics; a per-atom pass gathers each atom's
// own site share and its children's parent shares.
#include "pair.cuh"
#include "reduce.cuh"

#include <algorithm>
#include <cmath>

namespace t9gb {

constexpr float HAL_DELTA = 0.07f, HAL_GAMMA = 0.12f;

// reduced sites in slot order; w carries the van der Waals type
__global__ void k_vdw_pos(int npad, PairParams P, const int* __restrict__ perm, const float* __restrict__ xyz,
   const int* __restrict__ vtype, const int* __restrict__ vparent, const float* __restrict__ vred,
   float4* __restrict__ vpos)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      const int i = perm[s];
      if (i < 0) {
         vpos[s] = make_float4(0.f, 0.f, 0.f, __int_as_float(0));
         continue;
      }
      const int p = vparent[i];
      const float xi = xyz[3 * i], yi = xyz[3 * i + 1], zi = xyz[3 * i + 2];
      float4 v = make_float4(xi, yi, zi, __int_as_float(vtype[i]));
      if (p != i) {
         const float xp = xyz[3 * p], yp = xyz[3 * p + 1], zp = xyz[3 * p + 2];
         const float r = vred[i];
         v.x = xp + r * image1(xi - xp, P.lx, P.ilx);
         v.y = yp + r * image1(yi - yp, P.ly, P.ily);
         v.z = zp + r * image1(zi - zp, P.lz, P.ilz);
      }
      vpos[s] = v;
   }
}

// e and de/dr of one pair (pair_hal_v2 with vlambda = 1)
__device__ __forceinline__ void hal_pair(float r, float rv, float eps, float cut, float off, float& e, float& de)
{
   const float rinv = 1.f / rv;
   const float rho = r * rinv;
   const float rho6 = rho * rho * rho * rho * rho * rho;
   const float rho7 = rho6 * rho;
   const float rd = rho + HAL_DELTA;
   const float rd2 = rd * rd, rd3 = rd2 * rd, rd6 = rd3 * rd3;
   const float s1 = 1.f / (rd6 * rd);
   const float s2 = 1.f / (rho7 + HAL_GAMMA);
   const float c1 = 1.0f + HAL_DELTA;
   const float c12 = c1 * c1, c13 = c12 * c1;
   const float t1 = c13 * c13 * c1 * s1;
   const float t2 = (1.f + HAL_GAMMA) * s2;
   e = eps * t1 * (t2 - 2.f);
   const float dt1 = -7.f * rd6 * t1 * s1;
   const float dt2 = -7.f * rho6 * t2 * s2;
   de = eps * (dt1 * (t2 - 2.f) + t1 * dt2) * rinv;
   if (r > cut) {
      const float inv = 1.f / (cut - off);
      const float x = (r - off) * inv;
      const float x2 = x * x, x3 = x2 * x;
      const float taper = x3 * (6.f * x2 - 15.f * x + 10.f);
      const float dtaper = 30.f * (x * (1.f - x)) * (x * (1.f - x)) * inv;
      de = e * dtaper + de * taper;
      e *= taper;
   }
}

struct HalAcc {
   float e, g[3], w[9];
};

template <bool VIR>
__device__ __forceinline__ void hal_add(const PairParams& P, float4 a, float4 b, float vs, const float2* vtab, int nvt,
   float cut, float off2, float off, HalAcc& o)
{
   const float3 d = sep(P, a, b);
   const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
   if (r2 > off2 || vs == 0.f)
      return;
   const float2 t = vtab[__float_as_int(a.w) * nvt + __float_as_int(b.w)];
   const float r = sqrtf(r2);
   float e, de;
   hal_pair(r, t.x, t.y * vs, cut, off, e, de);
   const float dr = de / r;  // dE/dd = dr d, d = x_k - x_i
   o.e += 0.5f * e;
   o.g[0] -= dr * d.x;
   o.g[1] -= dr * d.y;
   o.g[2] -= dr * d.z;
   if (VIR) {
      const float dv[3] = {d.x, d.y, d.z};
#pragma unroll
      for (int p = 0; p < 3; ++p)
#pragma unroll
         for (int q = 0; q < 3; ++q)
            o.w[3 * p + q] += 0.5f * dr * dv[p] * dv[q];
   }
}

// G lanes per site: e_atom[s] (FP64), fout[s] = dE/dx of site s, virial rows
// wout[c][s] (may be null)
template <int G, bool VIR>
__global__ void __launch_bounds__(256) k_ehal(PairParams P, int npad, float cut, float off, const int* __restrict__ nbr,
   const int* __restrict__ nnbr, const int* __restrict__ sp_start, const int* __restrict__ sp_j,
   const float* __restrict__ sp_v, const float4* __restrict__ vpos, const float2* __restrict__ vtab, int nvt,
   double* __restrict__ e_atom, float* __restrict__ fout, float* __restrict__ wout)
{
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid / G, g = tid % G;
   if (i >= npad)
      return;
   HalAcc o;
   o.e = 0.f;
#pragma unroll
   for (int c = 0; c < 3; ++c)
      o.g[c] = 0.f;
#pragma unroll
   for (int c = 0; c < 9; ++c)
      o.w[c] = 0.f;
   const float off2 = off * off;
   if (i < P.n) {
      const float4 a = vpos[i];
      const int* row = nbr + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      for (int k = g; k < cnt; k += G)
         hal_add<VIR>(P, a, vpos[row[k]], 1.f, vtab, nvt, cut, off2, off, o);
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G)
         hal_add<VIR>(P, a, vpos[sp_j[q]], sp_v[q], vtab, nvt, cut, off2, off, o);
   }
   // FP32 lane sums of the FP32 lane partials (this GPU's FP64 pipe is far
   // narrower); the per-site energy is stored as FP64 for the FP64 total
   float acc[4] = {o.e, o.g[0], o.g[1], o.g[2]};
#pragma unroll
   for (int c = 0; c < 4; ++c)
#pragma unroll
      for (int s = G / 2; s > 0; s >>= 1)
         acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], s);
   float wv[9];
   if (VIR) {
#pragma unroll
      for (int c = 0; c < 9; ++c) {
         wv[c] = o.w[c];
#pragma unroll
         for (int s = G / 2; s > 0; s >>= 1)
            wv[c] += __shfl_xor_sync(0xffffffffu, wv[c], s);
      }
   }
   if (g == 0) {
      e_atom[i] = (double)acc[0];
      fout[3 * i] = acc[1];
      fout[3 * i + 1] = acc[2];
      fout[3 * i + 2] = acc[3];
      if (VIR)
#pragma unroll
         for (int c = 0; c < 9; ++c)
            wout[c * npad + i] = wv[c];
   }
}

// dE/dx of atom a (caller order): its own site's share plus its children's
// parent shares; add != 0 adds to grad
__global__ void k_vdw_combine(int n, const int* __restrict__ iperm, const int* __restrict__ vparent,
   const float* __restrict__ vred, const int* __restrict__ ch_start, const int* __restrict__ ch,
   const float* __restrict__ fsite, float* __restrict__ grad, int add)
{
   for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
      const float own = vparent[a] == a ? 1.f : vred[a];
      const float* f = fsite + 3 * iperm[a];
      float g[3] = {own * f[0], own * f[1], own * f[2]};
      for (int e = ch_start[a]; e < ch_start[a + 1]; ++e) {
         const int c = ch[e];
         const float w = 1.f - vred[c];
         const float* fc = fsite + 3 * iperm[c];
         g[0] += w * fc[0];
         g[1] += w * fc[1];
         g[2] += w * fc[2];
      }
      for (int c = 0; c < 3; ++c)
         grad[3 * a + c] = add ? grad[3 * a + c] + g[c] : g[c];
   }
}

// ---------------------------------------------------------------------------

static void vdw_free(Context* ctx)
{
   void* p[] = {ctx->vtab, ctx->vtype, ctx->vparent, ctx->vred, ctx->vch_start, ctx->vch, ctx->vpos, ctx->fvdw,
      ctx->e_vdw};
   for (void* q : p)
      if (q)
         cudaFree(q);
   ctx->vtab = nullptr;
   ctx->vtype = ctx->vparent = ctx->vch_start = ctx->vch = nullptr;
   ctx->vred = ctx->fvdw = nullptr;
   ctx->vpos = nullptr;
   ctx->e_vdw = nullptr;
}

void vdw_release(Context* ctx) { vdw_free(ctx); }

template <int G>
static void launch_ehal(Context* ctx, const PairParams& P, bool vir, double* ev, float* wv)
{
   const int nb = grid_for((long long)ctx->npad * G, 256);
   if (vir)
      k_ehal<G, true><<<nb, 256, 0, ctx->stream>>>(P, ctx->npad, (float)ctx->vdw_taper, (float)ctx->vdw_off,
         ctx->nbr, ctx->nnbr, ctx->sp_start, ctx->sp_j, ctx->sp_v, ctx->vpos, ctx->vtab, ctx->nvt, ev, ctx->fvdw, wv);
   else
      k_ehal<G, false><<<nb, 256, 0, ctx->stream>>>(P, ctx->npad, (float)ctx->vdw_taper, (float)ctx->vdw_off,
         ctx->nbr, ctx->nnbr, ctx->sp_start, ctx->sp_j, ctx->sp_v, ctx->vpos, ctx->vtab, ctx->nvt, ev, ctx->fvdw,
         nullptr);
}

int vdw_forces(Context* ctx, float* grad, bool add, bool vir, double* energy)
{
   if (!ctx->use_vdw)
      return T9GB_OK;
   PairParams P = make_params(ctx, ctx->vdw_off);
   k_vdw_pos<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, P, ctx->perm, ctx->xyz, ctx->vtype,
      ctx->vparent, ctx->vred, ctx->vpos);
   double* ev = ctx->e_vdw;  // every site's row written
   float* wv = vir ? ctx->wvir : nullptr;
   // lanes per atom: 16 on small boxes (more warps to hide the row loads),
   // 8 where the box fills the GPU anyway (GB300, ehal energy + gradient:
   // 12,288 atoms 0.123 / 0.133 ms at 16 / 8 lanes; 98,304 atoms 0.412 / 0.405)
   if (ctx->npad <= 32768)
      launch_ehal<16>(ctx, P, vir, ev, wv);
   else
      launch_ehal<8>(ctx, P, vir, ev, wv);
   if (grad)
      k_vdw_combine<<<grid_for(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, ctx->iperm, ctx->vparent, ctx->vred,
         ctx->vch_start, ctx->vch, ctx->fvdw, grad, add ? 1 : 0);
   T9_CUDA(cudaGetLastError());
   (void)energy;
   return T9GB_OK;
}

}  // namespace t9gb

using namespace t9gb;

extern "C" int t9gb_set_vdw(t9gb_context* h, int ntypes, const int* vtype, const double* radmin,
   const double* epsilon, const double* red, const int* parent, int nscaled, const int* scaled_ik,
   const double* scaled_v, double taper, double off)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_topology)
      return T9GB_NOT_READY;
   if (ntypes == 0) {
      vdw_free(ctx);
      ctx->use_vdw = false;
      ctx->have_order = false;
      drop_graphs(ctx);
      return T9GB_OK;
   }
   const int n = ctx->n;
   if (ntypes < 0 || ntypes > 256 || !vtype || !radmin || !epsilon || !red || !parent || nscaled < 0
      || (nscaled > 0 && (!scaled_ik || !scaled_v)) || !(off > 0) || !(taper >= 0) || taper > off
      || !std::isfinite(off))
      return T9GB_BAD_ARG;
   for (int i = 0; i < n; ++i) {
      if (vtype[i] < 0 || vtype[i] >= ntypes || parent[i] < 0 || parent[i] >= n || !std::isfinite(red[i])
         || red[i] < 0 || red[i] > 1)
         return T9GB_BAD_ARG;
   }
   std::vector<float2> tab((size_t)ntypes * ntypes);
   for (int a = 0; a < ntypes; ++a)
      for (int b = 0; b < ntypes; ++b) {
         const double r0 = radmin[(size_t)a * ntypes + b], e0 = epsilon[(size_t)a * ntypes + b];
         // each side of a pair reads its own row: the tables must be symmetric
         if (!(r0 > 0) || !std::isfinite(r0) || !(e0 >= 0) || !std::isfinite(e0)
            || r0 != radmin[(size_t)b * ntypes + a] || e0 != epsilon[(size_t)b * ntypes + a])
            return T9GB_BAD_ARG;
         tab[(size_t)a * ntypes + b] = make_float2((float)r0, (float)e0);
      }
   for (int j = 0; j < nscaled; ++j) {
      const int a = scaled_ik[2 * j], b = scaled_ik[2 * j + 1];
      if (a < 0 || b < 0 || a >= n || b >= n || a == b || !std::isfinite(scaled_v[j]))
         return T9GB_BAD_ARG;
   }
   // children of each atom (atoms reduced toward it), ascending
   std::vector<int> cstart(n + 1, 0), cl;
   std::vector<std::vector<int>> kids(n);
   for (int i = 0; i < n; ++i)
      if (parent[i] != i)
         kids[parent[i]].push_back(i);
   for (int i = 0; i < n; ++i) {
      cstart[i + 1] = cstart[i] + (int)kids[i].size();
      cl.insert(cl.end(), kids[i].begin(), kids[i].end());
   }
   vdw_free(ctx);
   std::vector<float> fred(red, red + n);
   for (int i = 0; i < n; ++i)
      fred[i] = parent[i] == i ? 0.f : (float)red[i];
   const size_t npad = ctx->npad;
   T9_CUDA(cudaMalloc(&ctx->vtab, sizeof(float2) * tab.size()));
   T9_CUDA(cudaMalloc(&ctx->vtype, sizeof(int) * n));
   T9_CUDA(cudaMalloc(&ctx->vparent, sizeof(int) * n));
   T9_CUDA(cudaMalloc(&ctx->vred, sizeof(float) * n));
   T9_CUDA(cudaMalloc(&ctx->vch_start, sizeof(int) * (n + 1)));
   T9_CUDA(cudaMalloc(&ctx->vch, sizeof(int) * std::max<size_t>(1, cl.size())));
   T9_CUDA(cudaMalloc(&ctx->vpos, sizeof(float4) * npad));
   T9_CUDA(cudaMalloc(&ctx->fvdw, sizeof(float) * 3 * npad));
   T9_CUDA(cudaMalloc(&ctx->e_vdw, sizeof(double) * npad));
   T9_CUDA(cudaMemcpy(ctx->vtab, tab.data(), sizeof(float2) * tab.size(), cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->vtype, vtype, sizeof(int) * n, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->vparent, parent, sizeof(int) * n, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->vred, fred.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->vch_start, cstart.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
   if (!cl.empty())
      T9_CUDA(cudaMemcpy(ctx->vch, cl.data(), sizeof(int) * cl.size(), cudaMemcpyHostToDevice));
   T9_CUDA(cudaDeviceSynchronize());
   ctx->nvt = ntypes;
   ctx->vdw_taper = taper;
   ctx->vdw_off = off;
   ctx->h_vtype.assign(vtype, vtype + n);
   ctx->h_vparent.assign(parent, parent + n);
   ctx->h_vred.assign(red, red + n);
   ctx->h_vexcl_ik.assign(scaled_ik, scaled_ik + 2 * (size_t)nscaled);
   ctx->h_vexcl_scale.assign(scaled_v, scaled_v + nscaled);
   ctx->use_vdw = true;
   // the stored list radius and the scaled-pair table change
   ctx->have_order = false;
   drop_graphs(ctx);
   return T9GB_OK;
}

extern "C" int t9gb_ehal(t9gb_context* h, int vers, double* energy, float* grad, double* virial)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
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
   if (!ctx->use_vdw) {
      ctx->last_error = "t9gb_ehal: no van der Waals parameters (t9gb_set_vdw)";
      return T9GB_NOT_READY;
   }
   const bool vir = (vers & T9GB_CALC_VIRIAL) != 0;
   T9_CHECK(force_setup(ctx));
   for (int attempt = 0; attempt < 2; ++attempt) {
      T9_CHECK(ensure_list(ctx));
      T9_CUDA(cudaMemsetAsync(ctx->e_atom, 0, sizeof(double) * 3 * ctx->npad, ctx->stream));
      T9_CHECK(vdw_forces(ctx, (vers & T9GB_CALC_GRAD) ? grad : nullptr, false, vir, nullptr));
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
      int redo = 0;
      T9_CHECK(check_list_overflow(ctx, &redo));
      if (!redo)
         break;
   }
   if (vers & T9GB_CALC_ENERGY)
      T9_CHECK(sum_rows_d(ctx, ctx->e_vdw, 1, energy));
   if (vir)
      T9_CHECK(sum_rows_virial(ctx, ctx->wvir, 1, virial));
   return T9GB_OK;
}
