// Sorted layout, scaled-partner table, per-step neighbour list, permutation
// and multipole-rotation kernels.
//
// The reference keeps atom arrays in input order and reaches them through
// SortedAtom::unsorted inside every pair kernel, with a 32x32 block-pair list
// rebuilt when atoms leave the list buffer (include/ff/spatial.h:15-140,
// src/cu/spatial.cu:149-960, src/spatial.cpp:201-205).  Here:
//  - the hot path lives in one spatial (Morton) order fixed when the order is
//    built; only the public entry points permute;
//  - every step (new coordinates) the device rebuilds an exact per-atom list
//    of neighbours within the cutoff from a cell grid (cells >= cutoff / 2,
//    5x5x5 stencil scanned as 25 contiguous x-runs), so the pair kernels
//    evaluate no pair beyond the cutoff and need no list buffer;
//  - scaled pairs (exclusions) are kept out of the list and evaluated from a
//    small per-atom partner table with their m/d/p/u scales, which is the
//    reference's exclusion-loop semantics (src/cu/amoeba/dfield_cu1.cc:30-106);
//  - list order is fixed (stencil order, then ascending slot within a cell),
//    so every real-space sum has a deterministic order.
#include <algorithm>
#include <cmath>
#include <map>

#include "common.cuh"

namespace t9gb {

static inline uint64_t spread_bits(uint64_t v)
{
   v &= 0x1fffff;
   v = (v | v << 32) & 0x1f00000000ffffULL;
   v = (v | v << 16) & 0x1f0000ff0000ffULL;
   v = (v | v << 8) & 0x100f00f00f00f00fULL;
   v = (v | v << 4) & 0x10c30c30c30c30c3ULL;
   v = (v | v << 2) & 0x1249249249249249ULL;
   return v;
}

static bool is_pbc(const t9gb_config& c) { return c.box[0] > 0 && c.box[1] > 0 && c.box[2] > 0; }

// The stored list holds the pairs within the largest per-step filter radius
// plus the list buffer: it is reused until an atom has moved more than half
// the buffer, so no pair inside a filter radius can be missing from it
// (neigh::lbuffer, src/nblist.cpp:312-530).
static double list_cutoff(const Context* ctx)
{
   const t9gb_config& c = ctx->cfg;
   double r = c.cutoff;
   if (c.pcgprec)
      r = std::max(r, c.usolve_cutoff + c.pbuffer);
   if (ctx->use_vdw)
      r = std::max(r, ctx->vdw_off + VDW_SITE_MARGIN);
   return r + std::max(0.0, c.list_buffer);
}

// Host: Morton order of the current coordinates, per-slot parameters, the
// scaled-partner table and the neighbour-list storage.
// the list and its two per-step sub-lists, all with row capacity cap
int alloc_lists(Context* ctx, int cap)
{
   for (int** p : {&ctx->nbr, &ctx->nbrc, &ctx->nbrp}) {
      cudaFree(*p);
      *p = nullptr;
      T9_CUDA(cudaMalloc(p, sizeof(int) * (size_t)ctx->npad * cap));
   }
   for (unsigned short** p : {&ctx->nbrc_l, &ctx->nbrp_l}) {
      cudaFree(*p);
      *p = nullptr;
      T9_CUDA(cudaMalloc(p, sizeof(unsigned short) * (size_t)ctx->npad * cap));
   }
   if (!ctx->jbl) {
      const int nblk = ctx->npad / 32;
      T9_CUDA(cudaMalloc(&ctx->jbl, sizeof(int) * (size_t)nblk * STAGE_JB_CAP));
      T9_CUDA(cudaMalloc(&ctx->jbn, sizeof(int) * (size_t)nblk));
      // no staging until a staging filter pass has written the lists
      T9_CUDA(cudaMemset(ctx->jbn, 0x7f, sizeof(int) * (size_t)nblk));
   }
   ctx->nbr_cap = cap;
   return T9GB_OK;
}

int order_build(Context* ctx)
{
   const int n = ctx->n, npad = ctx->npad;
   const t9gb_config& cfg = ctx->cfg;
   const bool pbc = is_pbc(cfg);
   const double* p = ctx->h_xyz.data();

   double lo[3], len[3];
   for (int d = 0; d < 3; ++d) {
      if (pbc) {
         lo[d] = 0;
         len[d] = cfg.box[d];
      } else {
         double mn = 1e300, mx = -1e300;
         for (int i = 0; i < n; ++i) {
            mn = std::min(mn, p[3 * i + d]);
            mx = std::max(mx, p[3 * i + d]);
         }
         lo[d] = mn;
         len[d] = std::max(mx - mn, 1.0);
      }
   }
   const double lmax = std::max(len[0], std::max(len[1], len[2]));
   int bits = 1;
   while ((1 << bits) * 1.5 < lmax && bits < 20)
      ++bits;
   const int g = 1 << bits;
   std::vector<std::pair<uint64_t, int>> key(n);
   for (int i = 0; i < n; ++i) {
      uint64_t c[3];
      for (int d = 0; d < 3; ++d) {
         double f = (p[3 * i + d] - lo[d]) / len[d];
         if (pbc)
            f -= std::floor(f);
         long v = (long)(f * g);
         v = std::min<long>(std::max<long>(v, 0), g - 1);
         c[d] = (uint64_t)v;
      }
      key[i] = {spread_bits(c[0]) | spread_bits(c[1]) << 1 | spread_bits(c[2]) << 2, i};
   }
   std::sort(key.begin(), key.end());
   ctx->h_perm.assign(npad, -1);
   ctx->h_iperm.assign(n, -1);
   for (int s = 0; s < n; ++s) {
      ctx->h_perm[s] = key[s].second;
      ctx->h_iperm[key[s].second] = s;
   }

   // scaled partners per slot, both directions, ascending partner slot: the
   // union of the electrostatic (m, d, p, u) and van der Waals scaled pairs,
   // each scale 1 where the other list does not name the pair
   struct Scales {
      float4 e;
      float v;
   };
   std::map<std::pair<int, int>, Scales> pairs;
   const int nex = (int)ctx->h_excl_scale.size() / 4;
   for (int j = 0; j < nex; ++j) {
      int a = ctx->h_excl_ik[2 * j], b = ctx->h_excl_ik[2 * j + 1];
      const double* v = &ctx->h_excl_scale[4 * j];
      pairs[{std::min(a, b), std::max(a, b)}] = {make_float4((float)v[0], (float)v[1], (float)v[2], (float)v[3]), 1.f};
   }
   if (ctx->use_vdw) {
      const int nv = (int)ctx->h_vexcl_scale.size();
      for (int j = 0; j < nv; ++j) {
         int a = ctx->h_vexcl_ik[2 * j], b = ctx->h_vexcl_ik[2 * j + 1];
         auto key = std::make_pair(std::min(a, b), std::max(a, b));
         auto it = pairs.find(key);
         if (it == pairs.end())
            pairs[key] = {make_float4(1.f, 1.f, 1.f, 1.f), (float)ctx->h_vexcl_scale[j]};
         else
            it->second.v = (float)ctx->h_vexcl_scale[j];
      }
   }
   struct Part {
      int k;
      float4 sc;
      float v;
   };
   std::vector<std::vector<Part>> part(npad);
   for (const auto& pr : pairs) {
      const int si = ctx->h_iperm[pr.first.first], sk = ctx->h_iperm[pr.first.second];
      part[si].push_back({sk, pr.second.e, pr.second.v});
      part[sk].push_back({si, pr.second.e, pr.second.v});
   }
   std::vector<int> sp_start(npad + 1, 0), sp_j;
   std::vector<float4> sp_sc;
   std::vector<float> sp_v;
   for (int s = 0; s < npad; ++s) {
      auto& v = part[s];
      std::sort(v.begin(), v.end(), [](const Part& a, const Part& b) { return a.k < b.k; });
      sp_start[s + 1] = sp_start[s] + (int)v.size();
      for (auto& e : v) {
         sp_j.push_back(e.k);
         sp_sc.push_back(e.sc);
         sp_v.push_back(e.v);
      }
   }
   ctx->nsp = (int)sp_j.size();

   // per-slot polarization parameters
   std::vector<float> pol(npad, 0.f), pinv(npad, 0.f);
   std::vector<float2> dmp(npad, make_float2(0.f, 0.f));
   for (int s = 0; s < n; ++s) {
      int a = ctx->h_perm[s];
      pol[s] = (float)ctx->h_polarity[a];
      pinv[s] = (float)(1.0 / std::max(ctx->h_polarity[a], 1.0e-16));
      const float tl = ctx->h_ptype.empty() ? (float)ctx->h_thole[a] : (float)ctx->h_ptype[a];
      dmp[s] = make_float2((float)ctx->h_pdamp[a], tl);
   }

   // cell grid and list capacity
   const double R = list_cutoff(ctx);
   ctx->list_cut = (float)R;
   ctx->use_cells = false;
   if (pbc && R < 1.0e6) {
      bool ok = true;
      for (int d = 0; d < 3; ++d) {
         ctx->nc[d] = (int)std::floor(cfg.box[d] / (0.5 * R * 1.0001));
         if (ctx->nc[d] < 5)
            ok = false;
      }
      ctx->use_cells = ok;
   }
   if (!ctx->use_cells && n > 16384) {
      ctx->last_error = "box too small for the cell grid (needs >= 2.5 cutoffs per edge) and too many atoms for "
                        "the all-pairs list";
      return T9GB_BAD_ARG;
   }
   int cap;
   if (ctx->use_cells) {
      ctx->ncell = ctx->nc[0] * ctx->nc[1] * ctx->nc[2];
      double vol = cfg.box[0] * cfg.box[1] * cfg.box[2];
      double expect = n / vol * 4.18879020478639 * R * R * R;
      cap = (int)(expect * 1.5) + 32;
   } else {
      ctx->ncell = 0;
      cap = npad;
   }
   cap = ((cap + 31) / 32) * 32;
   cap = std::max(cap, ctx->nbr_cap);

   cudaFree(ctx->perm);
   cudaFree(ctx->iperm);
   cudaFree(ctx->sp_start);
   cudaFree(ctx->sp_j);
   cudaFree(ctx->sp_sc);
   cudaFree(ctx->sp_v);
   ctx->sp_v = nullptr;
   cudaFree(ctx->cell_count);
   cudaFree(ctx->cell_start);
   ctx->perm = ctx->iperm = ctx->sp_start = ctx->sp_j = ctx->cell_count = ctx->cell_start = nullptr;
   ctx->sp_sc = nullptr;
   T9_CUDA(cudaMalloc(&ctx->perm, sizeof(int) * npad));
   T9_CUDA(cudaMalloc(&ctx->iperm, sizeof(int) * n));
   T9_CUDA(cudaMalloc(&ctx->sp_start, sizeof(int) * (npad + 1)));
   T9_CUDA(cudaMalloc(&ctx->sp_j, sizeof(int) * std::max(1, ctx->nsp)));
   T9_CUDA(cudaMalloc(&ctx->sp_sc, sizeof(float4) * std::max(1, ctx->nsp)));
   T9_CUDA(cudaMalloc(&ctx->sp_v, sizeof(float) * std::max(1, ctx->nsp)));
   T9_CUDA(cudaMemcpy(ctx->perm, ctx->h_perm.data(), sizeof(int) * npad, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->iperm, ctx->h_iperm.data(), sizeof(int) * n, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->sp_start, sp_start.data(), sizeof(int) * (npad + 1), cudaMemcpyHostToDevice));
   if (ctx->nsp) {
      T9_CUDA(cudaMemcpy(ctx->sp_j, sp_j.data(), sizeof(int) * ctx->nsp, cudaMemcpyHostToDevice));
      T9_CUDA(cudaMemcpy(ctx->sp_sc, sp_sc.data(), sizeof(float4) * ctx->nsp, cudaMemcpyHostToDevice));
      T9_CUDA(cudaMemcpy(ctx->sp_v, sp_v.data(), sizeof(float) * ctx->nsp, cudaMemcpyHostToDevice));
   }
   T9_CUDA(cudaMemcpy(ctx->spolar, pol.data(), sizeof(float) * npad, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->spolinv, pinv.data(), sizeof(float) * npad, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->sdamp, dmp.data(), sizeof(float2) * npad, cudaMemcpyHostToDevice));
   if (ctx->use_cells) {
      T9_CUDA(cudaMalloc(&ctx->cell_count, sizeof(int) * ctx->ncell));
      T9_CUDA(cudaMalloc(&ctx->cell_start, sizeof(int) * (ctx->ncell + 1)));
   }
   if (cap != ctx->nbr_cap)
      T9_CHECK(alloc_lists(ctx, cap));
   // legacy-stream copies above finish before the stream's kernels
   T9_CUDA(cudaDeviceSynchronize());
   T9_CHECK(fill_row_padding(ctx));
   T9_CHECK(frame_map_build(ctx));
   ctx->have_order = true;
   ctx->list_stale = true;
   ctx->list_need_build = true;
   drop_graphs(ctx);
   // a new order invalidates the predictor history
   return reset_predictor(ctx);
}

// Components 6 and 7 of every [npad][8] vector row hold the slot's thole and
// polarizability, so a neighbour's whole row is one 32-byte load.
__global__ void k_fill_pad(int npad, const float2* __restrict__ sdamp, const float* __restrict__ spolar,
   float* __restrict__ a)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      a[8 * s + 6] = sdamp[s].y;
      a[8 * s + 7] = spolar[s];
   }
}

int fill_row_padding(Context* ctx)
{
   float* rows[] = {ctx->rcp6, ctx->fld6, ctx->udir, ctx->efield, ctx->uind, ctx->rsd, ctx->zrsd, ctx->conj,
      ctx->vec, ctx->tmp6};
   for (float* a : rows)
      k_fill_pad<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, ctx->sdamp, ctx->spolar, a);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// ---------------------------------------------------------------------------
// device list build

struct CellParams {
   int n, npad;
   int ncx, ncy, ncz;
   float lx, ly, lz, ilx, ily, ilz;
   float r2;
   int cap;
};

__device__ __forceinline__ int cell_coord(float x, float il, int nc)
{
   float f = x * il;
   f -= floorf(f);
   int c = (int)(f * nc);
   return c < 0 ? 0 : (c >= nc ? nc - 1 : c);
}

__global__ void k_cell_assign(CellParams C, const float4* __restrict__ spos, int* __restrict__ atom_cell,
   int* __restrict__ cell_count)
{
   int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= C.n)
      return;
   float4 p = spos[s];
   int cx = cell_coord(p.x, C.ilx, C.ncx), cy = cell_coord(p.y, C.ily, C.ncy), cz = cell_coord(p.z, C.ilz, C.ncz);
   int c = (cz * C.ncy + cy) * C.ncx + cx;
   atom_cell[s] = c;
   atomicAdd(cell_count + c, 1);
}

// exclusive scan of the cell counts (one block); clears the counts for reuse
// as fill cursors
__global__ void k_cell_scan(int ncell, int* __restrict__ count, int* __restrict__ start)
{
   __shared__ int part[1024];
   const int t = threadIdx.x, nt = blockDim.x;
   const int chunk = (ncell + nt - 1) / nt;
   const int a = t * chunk, b = min(ncell, a + chunk);
   int sum = 0;
   for (int c = a; c < b; ++c)
      sum += count[c];
   part[t] = sum;
   __syncthreads();
   for (int o = 1; o < nt; o <<= 1) {
      int v = t >= o ? part[t - o] : 0;
      __syncthreads();
      part[t] += v;
      __syncthreads();
   }
   int run = part[t] - sum;
   for (int c = a; c < b; ++c) {
      start[c] = run;
      run += count[c];
      count[c] = 0;
   }
   if (t == nt - 1)
      start[ncell] = part[t];
}

__global__ void k_cell_fill(int n, const int* __restrict__ atom_cell, const int* __restrict__ start,
   int* __restrict__ cursor, int* __restrict__ cell_atoms)
{
   int s = blockIdx.x * blockDim.x + threadIdx.x;
   if (s >= n)
      return;
   int c = atom_cell[s];
   cell_atoms[start[c] + atomicAdd(cursor + c, 1)] = s;
}

// ascending slots inside each cell (fixes the list order): one warp per cell,
// each lane's rank is the count of smaller slots in the cell
__global__ void k_cell_sort(int ncell, const int* __restrict__ start, int* __restrict__ cell_atoms)
{
   const int c = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int lane = threadIdx.x & 31;
   if (c >= ncell)
      return;
   const int a = start[c], b = start[c + 1], cnt = b - a;
   if (cnt <= 32) {
      const int v = lane < cnt ? cell_atoms[a + lane] : 0x7fffffff;
      int rank = 0;
      for (int k = 0; k < 32; ++k)
         rank += __shfl_sync(0xffffffffu, v, k) < v ? 1 : 0;
      if (lane < cnt)
         cell_atoms[a + rank] = v;
   } else if (lane == 0) {
      for (int i = a + 1; i < b; ++i) {
         int v = cell_atoms[i];
         int j = i - 1;
         while (j >= a && cell_atoms[j] > v) {
            cell_atoms[j + 1] = cell_atoms[j];
            --j;
         }
         cell_atoms[j + 1] = v;
      }
   }
}

__device__ __forceinline__ bool is_partner(const int* __restrict__ sp_j, int a, int b, int j)
{
   for (int q = a; q < b; ++q)
      if (sp_j[q] == j)
         return true;
   return false;
}

// One warp per atom.  The 5x5x5 stencil is 25 x-rows of five consecutive
// cells, i.e. at most 50 contiguous runs of cell_atoms (a row splits in two
// where it wraps).  Lanes first record every run's start and length, then
// walk the concatenated candidate stream 32 at a time (a binary search maps a
// stream position to its run) and compact accepted neighbours with ballots,
// which keeps the list order fixed.
__global__ void __launch_bounds__(256) k_nbr_cells(CellParams C, const float4* __restrict__ spos,
   const int* __restrict__ atom_cell, const int* __restrict__ start, const int* __restrict__ cell_atoms,
   const int* __restrict__ sp_start, const int* __restrict__ sp_j, int* __restrict__ nbr, int* __restrict__ nnbr,
   int* __restrict__ over)
{
   __shared__ int s_off[8][52];
   __shared__ int s_beg[8][52];
   const int w = threadIdx.x >> 5;
   const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int lane = threadIdx.x & 31;
   if (i >= C.npad)
      return;
   if (i >= C.n) {
      if (lane == 0)
         nnbr[i] = 0;
      return;
   }
   const float4 pi = spos[i];
   const int ci = atom_cell[i];
   const int cix = ci % C.ncx, ciy = (ci / C.ncx) % C.ncy, ciz = ci / (C.ncx * C.ncy);
   int len[2], beg[2];
#pragma unroll
   for (int h = 0; h < 2; ++h) {
      const int r = lane + 32 * h;
      len[h] = 0;
      beg[h] = 0;
      if (r < 50) {
         const int q = r >> 1, part = r & 1;
         int cz = ciz + q / 5 - 2, cy = ciy + q % 5 - 2;
         cz += (cz < 0 ? C.ncz : 0) - (cz >= C.ncz ? C.ncz : 0);
         cy += (cy < 0 ? C.ncy : 0) - (cy >= C.ncy ? C.ncy : 0);
         const int row = (cz * C.ncy + cy) * C.ncx;
         const int x0 = cix - 2, x1 = cix + 2;
         int ca = 0, cb = -1;
         if (x0 < 0) {
            if (part == 0) {
               ca = x0 + C.ncx;
               cb = C.ncx - 1;
            } else {
               ca = 0;
               cb = x1;
            }
         } else if (x1 >= C.ncx) {
            if (part == 0) {
               ca = x0;
               cb = C.ncx - 1;
            } else {
               ca = 0;
               cb = x1 - C.ncx;
            }
         } else if (part == 0) {
            ca = x0;
            cb = x1;
         }
         if (cb >= ca) {
            beg[h] = start[row + ca];
            len[h] = start[row + cb + 1] - beg[h];
         }
      }
   }
   // exclusive offsets of the 64 run slots
   int inc0 = len[0], inc1 = len[1];
#pragma unroll
   for (int o = 1; o < 32; o <<= 1) {
      int v0 = __shfl_up_sync(0xffffffffu, inc0, o);
      int v1 = __shfl_up_sync(0xffffffffu, inc1, o);
      if (lane >= o) {
         inc0 += v0;
         inc1 += v1;
      }
   }
   const int tot0 = __shfl_sync(0xffffffffu, inc0, 31);
   const int total = tot0 + __shfl_sync(0xffffffffu, inc1, 31);
   s_off[w][lane] = inc0 - len[0];
   s_beg[w][lane] = beg[0];
   if (lane < 20) {
      s_off[w][32 + lane] = tot0 + inc1 - len[1];
      s_beg[w][32 + lane] = beg[1];
   }
   __syncwarp();
   const int pa = sp_start[i], pb = sp_start[i + 1];
   const unsigned lt = (1u << lane) - 1u;
   int* out = nbr + (size_t)i * C.cap;
   int cnt = 0;
   for (int t0 = 0; t0 < total; t0 += 32) {
      const int t = t0 + lane;
      bool acc = false;
      int j = -1;
      if (t < total) {
         int lo = 0, hi = 49;
         while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_off[w][mid] <= t)
               lo = mid;
            else
               hi = mid - 1;
         }
         j = cell_atoms[s_beg[w][lo] + (t - s_off[w][lo])];
         const float4 pj = spos[j];
         const float dx = image1(pj.x - pi.x, C.lx, C.ilx);
         const float dy = image1(pj.y - pi.y, C.ly, C.ily);
         const float dz = image1(pj.z - pi.z, C.lz, C.ilz);
         acc = j != i && dx * dx + dy * dy + dz * dz <= C.r2 && !is_partner(sp_j, pa, pb, j);
      }
      const unsigned m = __ballot_sync(0xffffffffu, acc);
      const int pos = cnt + __popc(m & lt);
      if (acc && pos < C.cap)
         out[pos] = j;
      cnt += __popc(m);
   }
   if (lane == 0) {
      nnbr[i] = min(cnt, C.cap);
      if (cnt > C.cap)
         atomicMax(over, cnt);
   }
}

// small or non-periodic systems: every slot is a candidate
__global__ void __launch_bounds__(256) k_nbr_all(CellParams C, const float4* __restrict__ spos,
   const int* __restrict__ sp_start, const int* __restrict__ sp_j, int* __restrict__ nbr, int* __restrict__ nnbr,
   int* __restrict__ over)
{
   const int i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
   const int lane = threadIdx.x & 31;
   if (i >= C.npad)
      return;
   if (i >= C.n) {
      if (lane == 0)
         nnbr[i] = 0;
      return;
   }
   const float4 pi = spos[i];
   const int pa = sp_start[i], pb = sp_start[i + 1];
   const unsigned lt = (1u << lane) - 1u;
   int cnt = 0;
   int* out = nbr + (size_t)i * C.cap;
   for (int t = 0; t < C.n; t += 32) {
      const int j = t + lane;
      bool acc = false;
      if (j < C.n && j != i) {
         float4 pj = spos[j];
         float dx = image1(pj.x - pi.x, C.lx, C.ilx);
         float dy = image1(pj.y - pi.y, C.ly, C.ily);
         float dz = image1(pj.z - pi.z, C.lz, C.ilz);
         acc = dx * dx + dy * dy + dz * dz <= C.r2 && !is_partner(sp_j, pa, pb, j);
      }
      const unsigned m = __ballot_sync(0xffffffffu, acc);
      const int pos = cnt + __popc(m & lt);
      if (acc && pos < C.cap)
         out[pos] = j;
      cnt += __popc(m);
   }
   if (lane == 0) {
      nnbr[i] = min(cnt, C.cap);
      if (cnt > C.cap)
         atomicMax(over, cnt);
   }
}

int list_update(Context* ctx)
{
   const t9gb_config& cfg = ctx->cfg;
   const bool pbc = is_pbc(cfg);
   CellParams C;
   C.n = ctx->n;
   C.npad = ctx->npad;
   C.ncx = ctx->nc[0];
   C.ncy = ctx->nc[1];
   C.ncz = ctx->nc[2];
   C.lx = pbc ? (float)cfg.box[0] : 0.f;
   C.ly = pbc ? (float)cfg.box[1] : 0.f;
   C.lz = pbc ? (float)cfg.box[2] : 0.f;
   C.ilx = pbc ? (float)(1.0 / cfg.box[0]) : 0.f;
   C.ily = pbc ? (float)(1.0 / cfg.box[1]) : 0.f;
   C.ilz = pbc ? (float)(1.0 / cfg.box[2]) : 0.f;
   double r2 = (double)ctx->list_cut * ctx->list_cut;
   C.r2 = r2 > 3.0e38 ? 3.0e38f : (float)r2;
   C.cap = ctx->nbr_cap;
   prof_begin(ctx, P_NBLIST);
   if (ctx->use_cells) {
      T9_CUDA(cudaMemsetAsync(ctx->cell_count, 0, sizeof(int) * ctx->ncell, ctx->stream));
      k_cell_assign<<<grid_for(ctx->n, 256), 256, 0, ctx->stream>>>(C, ctx->spos, ctx->atom_cell, ctx->cell_count);
      k_cell_scan<<<1, 1024, 0, ctx->stream>>>(ctx->ncell, ctx->cell_count, ctx->cell_start);
      k_cell_fill<<<grid_for(ctx->n, 256), 256, 0, ctx->stream>>>(ctx->n, ctx->atom_cell, ctx->cell_start,
         ctx->cell_count, ctx->cell_atoms);
      k_cell_sort<<<grid_for((long long)ctx->ncell * 32, 256), 256, 0, ctx->stream>>>(ctx->ncell, ctx->cell_start,
         ctx->cell_atoms);
      k_nbr_cells<<<grid_for((long long)ctx->npad * 32, 256), 256, 0, ctx->stream>>>(C, ctx->spos, ctx->atom_cell,
         ctx->cell_start, ctx->cell_atoms, ctx->sp_start, ctx->sp_j, ctx->nbr, ctx->nnbr, ctx->nbr_over);
   } else {
      k_nbr_all<<<grid_for((long long)ctx->npad * 32, 256), 256, 0, ctx->stream>>>(C, ctx->spos, ctx->sp_start,
         ctx->sp_j, ctx->nbr, ctx->nnbr, ctx->nbr_over);
   }
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// ---------------------------------------------------------------------------
// positions and permutations

// sorted positions, w = pdamp (read with the position by every pair kernel)
__global__ void k_scatter_pos(int npad, const int* __restrict__ perm, const float* __restrict__ xyz,
   const float2* __restrict__ sdamp, float4* __restrict__ spos)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      int a = perm[s];
      float4 v = make_float4(0.f, 0.f, 0.f, 0.f);
      if (a >= 0)
         v = make_float4(xyz[3 * a], xyz[3 * a + 1], xyz[3 * a + 2], sdamp[s].x);
      spos[s] = v;
   }
}

int scatter_positions(Context* ctx)
{
   k_scatter_pos<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, ctx->perm, ctx->xyz, ctx->sdamp,
      ctx->spos);
   T9_CUDA(cudaGetLastError());
   ctx->list_stale = true;
   return T9GB_OK;
}

// caller-order [n][3] pair -> sorted rows of 8 (components 6, 7 untouched)
__global__ void k_gather6(int npad, const int* __restrict__ perm, const float* __restrict__ a,
   const float* __restrict__ b, float* __restrict__ s8)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      int at = perm[s];
      float v[6] = {0, 0, 0, 0, 0, 0};
      if (at >= 0) {
         for (int d = 0; d < 3; ++d) {
            v[d] = a[3 * at + d];
            v[3 + d] = b ? b[3 * at + d] : 0.f;
         }
      }
      for (int d = 0; d < 6; ++d)
         s8[8 * s + d] = v[d];
   }
}

int gather_to_sorted3(Context* ctx, const float* a, const float* b, float* s6)
{
   k_gather6<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, ctx->perm, a, b, s6);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

__global__ void k_scatter6(int npad, const int* __restrict__ perm, const float* __restrict__ s6, float* __restrict__ a,
   float* __restrict__ b)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      int at = perm[s];
      if (at < 0)
         continue;
      for (int d = 0; d < 3; ++d) {
         if (a)
            a[3 * at + d] = s6[8 * s + d];
         if (b)
            b[3 * at + d] = s6[8 * s + 3 + d];
      }
   }
}

int scatter_from_sorted3(Context* ctx, const float* s6, float* a, float* b)
{
   k_scatter6<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, ctx->perm, s6, a, b);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// ---------------------------------------------------------------------------
// multipole rotation (include/seq/rotpole.h:7-224), sorted output

__device__ __forceinline__ void norm3(float* a)
{
   float r = rsqrtf(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
   a[0] *= r;
   a[1] *= r;
   a[2] *= r;
}

// chirality check (rotpole.h:7-50): flips y-odd components once, in place
__device__ __forceinline__ void chkpole_one(int i, int4* __restrict__ frames, float* __restrict__ pole,
   const float* __restrict__ xyz)
{
   {
      int4 f = frames[i];
      if (f.w != 2 || f.z == 0)
         return;
      int id = abs(f.z) - 1;
      const float* pa = xyz + 3 * i;
      const float* pb = xyz + 3 * f.x;
      const float* pc = xyz + 3 * f.y;
      const float* pd = xyz + 3 * id;
      float xad = pa[0] - pd[0], yad = pa[1] - pd[1], zad = pa[2] - pd[2];
      float xbd = pb[0] - pd[0], ybd = pb[1] - pd[1], zbd = pb[2] - pd[2];
      float xcd = pc[0] - pd[0], ycd = pc[1] - pd[1], zcd = pc[2] - pd[2];
      float c1 = ybd * zcd - zbd * ycd, c2 = ycd * zad - zcd * yad, c3 = yad * zbd - zad * ybd;
      float vol = xad * c1 + xbd * c2 + xcd * c3;
      if ((f.z < 0 && vol > 0) || (f.z > 0 && vol < 0)) {
         frames[i].z = -f.z;
         pole[10 * i + 2] = -pole[10 * i + 2];
         pole[10 * i + 7] = -pole[10 * i + 7];
         pole[10 * i + 9] = -pole[10 * i + 9];
      }
   }
}

// rows of 12: q, d xyz, qxx, qyy, qzz, qxy, qxz, qyz, thole, polarizability
// also stores the local frame (rows x, y, z axes) per slot in sframe[9]
// The chirality check of the slot's own atom runs first (chkpole): the
// thread is the only one touching that atom, and it reads back what it wrote.
__global__ void k_rotpole(int npad, const int* __restrict__ perm, int4* __restrict__ frames, float* __restrict__ pole,
   const float* __restrict__ xyz, const float2* __restrict__ sdamp, const float* __restrict__ spolar,
   float* __restrict__ rpole, float* __restrict__ sframe)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      int i = perm[s];
      float* rp = rpole + 12 * s;
      float* fr = sframe + 9 * s;
      if (i < 0) {
         for (int c = 0; c < 12; ++c)
            rp[c] = 0.f;
         for (int c = 0; c < 9; ++c)
            fr[c] = (c % 4 == 0) ? 1.f : 0.f;
         continue;
      }
      chkpole_one(i, frames, pole, xyz);
      rp[10] = sdamp[s].y;
      rp[11] = spolar[s];
      int4 f = frames[i];
      float a[3][3] = {{1, 0, 0}, {0, 1, 0}, {0, 0, 1}};
      if (f.w != 0) {
         float xi = xyz[3 * i], yi = xyz[3 * i + 1], zi = xyz[3 * i + 2];
         float* xx = a[0];
         float* yy = a[1];
         float* zz = a[2];
         zz[0] = xyz[3 * f.x] - xi;
         zz[1] = xyz[3 * f.x + 1] - yi;
         zz[2] = xyz[3 * f.x + 2] - zi;
         norm3(zz);
         if (f.w == 1) {
            bool okay = !(fabsf(zz[0]) > 0.866f);
            xx[0] = okay ? 1.f : 0.f;
            xx[1] = okay ? 0.f : 1.f;
            xx[2] = 0.f;
         } else {
            xx[0] = xyz[3 * f.y] - xi;
            xx[1] = xyz[3 * f.y + 1] - yi;
            xx[2] = xyz[3 * f.y + 2] - zi;
            norm3(xx);
         }
         if (f.w == 4 || f.w == 5) {
            int iy = abs(f.z) - 1;
            yy[0] = xyz[3 * iy] - xi;
            yy[1] = xyz[3 * iy + 1] - yi;
            yy[2] = xyz[3 * iy + 2] - zi;
            norm3(yy);
         }
         if (f.w == 3) {
            for (int d = 0; d < 3; ++d)
               zz[d] += xx[d];
            norm3(zz);
         } else if (f.w == 4) {
            for (int d = 0; d < 3; ++d)
               xx[d] += yy[d];
            norm3(xx);
         } else if (f.w == 5) {
            for (int d = 0; d < 3; ++d)
               zz[d] += xx[d] + yy[d];
            norm3(zz);
         }
         float dot = xx[0] * zz[0] + xx[1] * zz[1] + xx[2] * zz[2];
         for (int d = 0; d < 3; ++d)
            xx[d] -= dot * zz[d];
         norm3(xx);
         a[1][0] = a[0][2] * a[2][1] - a[0][1] * a[2][2];
         a[1][1] = a[0][0] * a[2][2] - a[0][2] * a[2][0];
         a[1][2] = a[0][1] * a[2][0] - a[0][0] * a[2][1];
      }
      for (int r = 0; r < 3; ++r)
         for (int c = 0; c < 3; ++c)
            fr[3 * r + c] = a[r][c];
      const float* p = pole + 10 * i;
      rp[0] = p[0];
      for (int c = 0; c < 3; ++c)
         rp[1 + c] = p[1] * a[0][c] + p[2] * a[1][c] + p[3] * a[2][c];
      float mp[3][3] = {{p[4], p[7], p[8]}, {p[7], p[5], p[9]}, {p[8], p[9], p[6]}};
      float q[3][3];
      for (int c = 0; c < 3; ++c)
         for (int j = 0; j <= c; ++j) {
            float acc = 0.f;
            for (int k = 0; k < 3; ++k)
               for (int m = 0; m < 3; ++m)
                  acc += a[k][c] * a[m][j] * mp[m][k];
            q[j][c] = acc;
         }
      rp[4] = q[0][0];
      rp[5] = q[1][1];
      rp[6] = q[2][2];
      rp[7] = q[0][1];
      rp[8] = q[0][2];
      rp[9] = q[1][2];
   }
}

int rotpole_sorted(Context* ctx)
{
   k_rotpole<<<grid_for(ctx->npad, 128), 128, 0, ctx->stream>>>(ctx->npad, ctx->perm, ctx->frames, ctx->pole,
      ctx->xyz, ctx->sdamp, ctx->spolar, ctx->srpole, ctx->sframe);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

}  // namespace t9gb
