// Bond, angle and Urey-Bradley terms of the MD step around induce().
//
// Restates the reference's harmonic valence kernels (include/seq/bond.h:44-59
// anharmonic bond with bond-cubic / bond-quartic, include/seq/angle.h:88-150
// HARMONIC angle in degrees with angle-cubic ... angle-sextic,
// include/seq/urey.h:44-60 Urey-Bradley 1-3 distance with urey-cubic /
// urey-quartic; bondunit 1, angunit (pi/180)^2, ureyunit 1).  One thread per
// term writes the gradient on each of its atoms to a per-term slot; a
// per-atom pass sums an atom's slots through a fixed CSR order, so the
// gradient needs no atomics and is bit-reproducible.
#include "pair.cuh"

#include <algorithm>
#include <cmath>

namespace t9gb {

struct ValParams {
   float cbnd, qbnd;              // bond cubic, quartic
   float cang, qang, pang, sang;  // angle cubic ... sextic
   float cury, qury;              // Urey-Bradley cubic, quartic
   float lx, ly, lz, ilx, ily, ilz;
};

__device__ __forceinline__ float3 vsub(const ValParams& V, const float* xyz, int a, int b)
{
   return make_float3(image1(xyz[3 * a] - xyz[3 * b], V.lx, V.ilx), image1(xyz[3 * a + 1] - xyz[3 * b + 1], V.ly, V.ily),
      image1(xyz[3 * a + 2] - xyz[3 * b + 2], V.lz, V.ilz));
}

// term t: idx = (a, b, c, kind) with kind 0 bond (a, b), 1 angle (a, vertex b,
// c), 2 Urey-Bradley (a, vertex b, c; the a-c distance); par = (k, ideal).
// Outputs: g[t][3 roles][3], e[t], and with VIR the virial rows w[9][nterm].
template <bool VIR>
__global__ void k_valence(int nterm, ValParams V, const int4* __restrict__ idx, const float2* __restrict__ par,
   const float* __restrict__ xyz, float* __restrict__ g, double* __restrict__ e, float* __restrict__ w)
{
   constexpr float RAD = 57.29577951308232f;  // degrees per radian
   constexpr float ANGUNIT = 1.f / (RAD * RAD);
   for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < nterm; t += gridDim.x * blockDim.x) {
      const int4 q = idx[t];
      const float2 p = par[t];
      float ga[3] = {0, 0, 0}, gb[3] = {0, 0, 0}, gc[3] = {0, 0, 0};
      float en = 0.f;
      float3 ra = make_float3(0, 0, 0), rc = make_float3(0, 0, 0);  // positions relative to b
      if (q.w == 0 || q.w == 2) {
         // bond a-b, or the Urey-Bradley a-c distance
         const int j = q.w == 0 ? q.y : q.z;
         const float3 d = vsub(V, xyz, q.x, j);
         const float r = sqrtf(d.x * d.x + d.y * d.y + d.z * d.z);
         const float dt = r - p.y, dt2 = dt * dt;
         const float c3 = q.w == 0 ? V.cbnd : V.cury, c4 = q.w == 0 ? V.qbnd : V.qury;
         en = p.x * dt2 * (1.f + c3 * dt + c4 * dt2);
         const float de = 2.f * p.x * dt * (1.f + 1.5f * c3 * dt + 2.f * c4 * dt2) / r;
         ga[0] = de * d.x;
         ga[1] = de * d.y;
         ga[2] = de * d.z;
         float* gj = q.w == 0 ? gb : gc;
         gj[0] = -ga[0];
         gj[1] = -ga[1];
         gj[2] = -ga[2];
         if (q.w == 0)
            ra = d;
         else {
            ra = vsub(V, xyz, q.x, q.y);
            rc = vsub(V, xyz, q.z, q.y);
         }
      } else {
         // angle a-b-c at vertex b
         ra = vsub(V, xyz, q.x, q.y);
         rc = vsub(V, xyz, q.z, q.y);
         const float ra2 = ra.x * ra.x + ra.y * ra.y + ra.z * ra.z;
         const float rc2 = rc.x * rc.x + rc.y * rc.y + rc.z * rc.z;
         if (ra2 != 0.f && rc2 != 0.f) {
            float cs = (ra.x * rc.x + ra.y * rc.y + ra.z * rc.z) * rsqrtf(ra2 * rc2);
            cs = fminf(1.f, fmaxf(-1.f, cs));
            const float dt = RAD * acosf(cs) - p.y;
            const float dt2 = dt * dt, dt3 = dt2 * dt, dt4 = dt2 * dt2;
            en = ANGUNIT * p.x * dt2 * (1.f + V.cang * dt + V.qang * dt2 + V.pang * dt3 + V.sang * dt4);
            // dE/dtheta (per radian)
            const float det = ANGUNIT * p.x * dt * RAD
               * (2.f + 3.f * V.cang * dt + 4.f * V.qang * dt2 + 5.f * V.pang * dt3 + 6.f * V.sang * dt4);
            // n = rc x ra; dtheta/dx_a = (ra x n) / (|ra|^2 |n|), dtheta/dx_c = -(rc x n) / (|rc|^2 |n|)
            const float nx = rc.y * ra.z - rc.z * ra.y, ny = rc.z * ra.x - rc.x * ra.z, nz = rc.x * ra.y - rc.y * ra.x;
            const float nn = fmaxf(sqrtf(nx * nx + ny * ny + nz * nz), 1e-6f);
            const float fa = -det / (ra2 * nn), fc = det / (rc2 * nn);
            ga[0] = fa * (ra.y * nz - ra.z * ny);
            ga[1] = fa * (ra.z * nx - ra.x * nz);
            ga[2] = fa * (ra.x * ny - ra.y * nx);
            gc[0] = fc * (rc.y * nz - rc.z * ny);
            gc[1] = fc * (rc.z * nx - rc.x * nz);
            gc[2] = fc * (rc.x * ny - rc.y * nx);
            for (int k = 0; k < 3; ++k)
               gb[k] = -ga[k] - gc[k];
         }
      }
      float* o = g + 9 * (size_t)t;
      for (int k = 0; k < 3; ++k) {
         o[k] = ga[k];
         o[3 + k] = gb[k];
         o[6 + k] = gc[k];
      }
      e[t] = en;
      if (VIR) {
         // dE/d(eps_ab) = sum over atoms of g_a x_b, positions relative to b
         const float xa[3] = {ra.x, ra.y, ra.z}, xc[3] = {rc.x, rc.y, rc.z};
         for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
               w[(3 * a + b) * (size_t)nterm + t] = ga[a] * xa[b] + gc[a] * xc[b];
      }
   }
}

// per-atom sum of its term slots (entry = 3 term + role), added to grad
__global__ void k_valence_gather(int n, const int* __restrict__ start, const int* __restrict__ ent,
   const float* __restrict__ g, float* __restrict__ grad, int add)
{
   for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
      float s[3] = {0.f, 0.f, 0.f};
      for (int e = start[a]; e < start[a + 1]; ++e) {
         const float* f = g + 3 * (size_t)ent[e];
         s[0] += f[0];
         s[1] += f[1];
         s[2] += f[2];
      }
      for (int c = 0; c < 3; ++c)
         grad[3 * a + c] = add ? grad[3 * a + c] + s[c] : s[c];
   }
}

// block b sums rows[b][0..m) (FP64 out[b]); one block per row
__global__ void k_rows_sum(int m, const float* __restrict__ rows, const double* __restrict__ drow,
   double* __restrict__ out)
{
   __shared__ double sh[256];
   double v = 0;
   for (int i = threadIdx.x; i < m; i += blockDim.x)
      v += drow ? drow[i] : (double)rows[(size_t)blockIdx.x * m + i];
   sh[threadIdx.x] = v;
   __syncthreads();
   for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o)
         sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
   }
   if (threadIdx.x == 0)
      out[blockIdx.x] = sh[0];
}

static void val_free(Context* ctx)
{
   void* p[] = {ctx->val_idx, ctx->val_par, ctx->val_g, ctx->val_e, ctx->val_w, ctx->val_start, ctx->val_ent,
      ctx->val_sum};
   for (void* q : p)
      if (q)
         cudaFree(q);
   ctx->val_idx = nullptr;
   ctx->val_par = nullptr;
   ctx->val_g = ctx->val_w = nullptr;
   ctx->val_e = ctx->val_sum = nullptr;
   ctx->val_start = ctx->val_ent = nullptr;
   ctx->nval = 0;
}

void valence_release(Context* ctx) { val_free(ctx); }

static ValParams val_params(const Context* ctx)
{
   ValParams V;
   const double* g = ctx->val_glob;
   V.cbnd = (float)g[0];
   V.qbnd = (float)g[1];
   V.cang = (float)g[2];
   V.qang = (float)g[3];
   V.pang = (float)g[4];
   V.sang = (float)g[5];
   V.cury = (float)g[6];
   V.qury = (float)g[7];
   const bool pbc = ctx->cfg.box[0] > 0 && ctx->cfg.box[1] > 0 && ctx->cfg.box[2] > 0;
   V.lx = pbc ? (float)ctx->cfg.box[0] : 0.f;
   V.ly = pbc ? (float)ctx->cfg.box[1] : 0.f;
   V.lz = pbc ? (float)ctx->cfg.box[2] : 0.f;
   V.ilx = pbc ? (float)(1.0 / ctx->cfg.box[0]) : 0.f;
   V.ily = pbc ? (float)(1.0 / ctx->cfg.box[1]) : 0.f;
   V.ilz = pbc ? (float)(1.0 / ctx->cfg.box[2]) : 0.f;
   return V;
}

// valence gradient into grad (added when add), energy terms in val_e,
// virial rows in val_w when vir
int valence_forces(Context* ctx, float* grad, bool add, bool vir)
{
   if (ctx->nval == 0)
      return T9GB_OK;
   const ValParams V = val_params(ctx);
   const int nb = grid_for(ctx->nval, 256);
   if (vir)
      k_valence<true><<<nb, 256, 0, ctx->stream>>>(ctx->nval, V, ctx->val_idx, ctx->val_par, ctx->xyz, ctx->val_g,
         ctx->val_e, ctx->val_w);
   else
      k_valence<false><<<nb, 256, 0, ctx->stream>>>(ctx->nval, V, ctx->val_idx, ctx->val_par, ctx->xyz, ctx->val_g,
         ctx->val_e, nullptr);
   if (grad)
      k_valence_gather<<<grid_for(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, ctx->val_start, ctx->val_ent,
         ctx->val_g, grad, add ? 1 : 0);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// energy (and virial) sums of the last valence_forces: host doubles
int valence_sums(Context* ctx, double* energy, double* virial)
{
   if (ctx->nval == 0) {
      if (energy)
         *energy = 0;
      if (virial)
         for (int c = 0; c < 9; ++c)
            virial[c] = 0;
      return T9GB_OK;
   }
   k_rows_sum<<<1, 256, 0, ctx->stream>>>(ctx->nval, nullptr, ctx->val_e, ctx->val_sum);
   if (virial)
      k_rows_sum<<<9, 256, 0, ctx->stream>>>(ctx->nval, ctx->val_w, nullptr, ctx->val_sum + 1);
   T9_CUDA(cudaGetLastError());
   double h[10];
   T9_CUDA(cudaMemcpyAsync(h, ctx->val_sum, sizeof(double) * 10, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   if (energy)
      *energy = h[0];
   if (virial)
      for (int a = 0; a < 3; ++a)
         for (int b = 0; b < 3; ++b)
            virial[3 * a + b] = 0.5 * (h[1 + 3 * a + b] + h[1 + 3 * b + a]);
   return T9GB_OK;
}

}  // namespace t9gb

using namespace t9gb;

extern "C" int t9gb_set_valence(t9gb_context* h, int nbond, const int* ibnd, const double* bk, const double* bl,
   double cbnd, double qbnd, int nangle, const int* iang, const double* ak, const double* anat, const double* angle_terms,
   int nurey, const int* iury, const double* uk, const double* ul, double cury, double qury)
{
   if (!h || nbond < 0 || nangle < 0 || nurey < 0)
      return T9GB_BAD_ARG;
   if ((nbond && (!ibnd || !bk || !bl)) || (nangle && (!iang || !ak || !anat || !angle_terms))
      || (nurey && (!iury || !uk || !ul)))
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   const int n = ctx->n;
   const int nt = nbond + nangle + nurey;
   std::vector<int4> idx(nt);
   std::vector<float2> par(nt);
   auto ok = [n](int a) { return a >= 0 && a < n; };
   for (int j = 0; j < nbond; ++j) {
      const int a = ibnd[2 * j], b = ibnd[2 * j + 1];
      if (!ok(a) || !ok(b) || a == b || !std::isfinite(bk[j]) || !(bl[j] > 0))
         return T9GB_BAD_ARG;
      idx[j] = make_int4(a, b, -1, 0);
      par[j] = make_float2((float)bk[j], (float)bl[j]);
   }
   for (int j = 0; j < nangle; ++j) {
      const int a = iang[3 * j], b = iang[3 * j + 1], c = iang[3 * j + 2];
      if (!ok(a) || !ok(b) || !ok(c) || a == b || b == c || a == c || !std::isfinite(ak[j]) || !std::isfinite(anat[j]))
         return T9GB_BAD_ARG;
      idx[nbond + j] = make_int4(a, b, c, 1);
      par[nbond + j] = make_float2((float)ak[j], (float)anat[j]);
   }
   for (int j = 0; j < nurey; ++j) {
      const int a = iury[3 * j], b = iury[3 * j + 1], c = iury[3 * j + 2];
      if (!ok(a) || !ok(b) || !ok(c) || a == c || !std::isfinite(uk[j]) || !(ul[j] > 0))
         return T9GB_BAD_ARG;
      idx[nbond + nangle + j] = make_int4(a, b, c, 2);
      par[nbond + nangle + j] = make_float2((float)uk[j], (float)ul[j]);
   }
   // per-atom CSR of (term, role) slots, terms ascending
   std::vector<std::vector<int>> per(n);
   for (int t = 0; t < nt; ++t) {
      per[idx[t].x].push_back(3 * t);
      per[idx[t].y].push_back(3 * t + 1);
      if (idx[t].w != 0)
         per[idx[t].z].push_back(3 * t + 2);
   }
   std::vector<int> start(n + 1, 0), ent;
   for (int a = 0; a < n; ++a) {
      start[a + 1] = start[a] + (int)per[a].size();
      ent.insert(ent.end(), per[a].begin(), per[a].end());
   }
   val_free(ctx);
   const double glob[8] = {cbnd, qbnd, nangle ? angle_terms[0] : 0.0, nangle ? angle_terms[1] : 0.0,
      nangle ? angle_terms[2] : 0.0, nangle ? angle_terms[3] : 0.0, cury, qury};
   for (int c = 0; c < 8; ++c) {
      if (!std::isfinite(glob[c]))
         return T9GB_BAD_ARG;
      ctx->val_glob[c] = glob[c];
   }
   if (nt == 0)
      return T9GB_OK;
   T9_CUDA(cudaMalloc(&ctx->val_idx, sizeof(int4) * nt));
   T9_CUDA(cudaMalloc(&ctx->val_par, sizeof(float2) * nt));
   T9_CUDA(cudaMalloc(&ctx->val_g, sizeof(float) * 9 * (size_t)nt));
   T9_CUDA(cudaMalloc(&ctx->val_e, sizeof(double) * nt));
   T9_CUDA(cudaMalloc(&ctx->val_w, sizeof(float) * 9 * (size_t)nt));
   T9_CUDA(cudaMalloc(&ctx->val_start, sizeof(int) * (n + 1)));
   T9_CUDA(cudaMalloc(&ctx->val_ent, sizeof(int) * std::max<size_t>(1, ent.size())));
   T9_CUDA(cudaMalloc(&ctx->val_sum, sizeof(double) * 10));
   T9_CUDA(cudaMemcpy(ctx->val_idx, idx.data(), sizeof(int4) * nt, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->val_par, par.data(), sizeof(float2) * nt, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->val_start, start.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice));
   if (!ent.empty())
      T9_CUDA(cudaMemcpy(ctx->val_ent, ent.data(), sizeof(int) * ent.size(), cudaMemcpyHostToDevice));
   T9_CUDA(cudaDeviceSynchronize());
   ctx->nval = nt;
   return T9GB_OK;
}

extern "C" int t9gb_evalence(t9gb_context* h, int vers, double* energy, float* grad, double* virial)
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
   if (!ctx->have_xyz)
      return T9GB_NOT_READY;
   const bool vir = (vers & T9GB_CALC_VIRIAL) != 0;
   T9_CHECK(valence_forces(ctx, (vers & T9GB_CALC_GRAD) ? grad : nullptr, false, vir));
   if ((vers & T9GB_CALC_GRAD) && ctx->nval == 0)
      T9_CUDA(cudaMemsetAsync(grad, 0, sizeof(float) * 3 * ctx->n, ctx->stream));
   double e = 0;
   T9_CHECK(valence_sums(ctx, &e, vir ? virial : nullptr));
   if (energy)
      *energy = e;
   return T9GB_OK;
}
