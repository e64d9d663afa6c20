// Real-space pair kernels over the per-step neighbour list.
//
// G consecutive lanes own one atom i (t9gb_pair_lanes: 8 up to 32,768 atoms,
// 4 above): lane g walks the list entries g, g+G, g+2G, ... of atom i
// (consecutive addresses per step, two entries in flight per trip), then the
// scaled partners of i the same way; the partial fields are combined with a
// fixed xor-shuffle tree and written with plain stores.  Every pair is
// evaluated from both sides (full list), so no atomics are needed and each
// field component is a sum in a fixed order: results are bit-reproducible.
// 12,288 atoms at 8 lanes give 98,304 threads, ~20 warps on each of the 152
// SMs.
//
// Pair arithmetic restates the reference's pair_dfield_v2 / pair_ufield_v2
// (include/seq/pair_field.h:127-256, :333-420) for the atom-i side, Thole
// damping damp_thole2/3 (include/seq/damp.h:8-44), the Ewald b_n recursion
// damp_ewald (include/seq/damp.h:136-151), and the preconditioner pair of
// sparsePrecond_cu1 (src/cu/amoeba/sparsePrecond_cu1.cc:60-120).  The k side
// of the reference's pair functions equals the i-side formula evaluated from
// atom k with the separation reversed, which is what the full list does.
#include "pair.cuh"
#include "reduce.cuh"

namespace t9gb {


__device__ __forceinline__ void thole_damp(float r, float pdi, float pgamma, float pdk, float& s3, float& s5,
   float& s7)
{
   float damp = pdi * pdk;
   float ratio = r * __frcp_rn(damp);
   damp = (damp == 0.f) ? -1.0e16f : -pgamma * ratio * ratio * ratio;
   float ex = __expf(damp);
   s3 = 1.f - ex;
   s5 = 1.f - ex * (1.f - damp);
   s7 = 1.f - ex * (1.f - damp + 0.6f * damp * damp);
}

__device__ __forceinline__ void ewald_bn(const PairParams& P, float r, float invr, float rr2, float& b1, float& b2,
   float& b3)
{
   float ralpha = P.aewald * r;
   float exp2a = __expf(-ralpha * ralpha);
   float b0 = erfc_hastings(ralpha, exp2a) * invr;
   b1 = (b0 + P.ec1 * exp2a) * rr2;
   b2 = (3.f * b1 + P.ec2 * exp2a) * rr2;
   b3 = (5.f * b2 + P.ec3 * exp2a) * rr2;
}




__device__ __forceinline__ float pick6(const float* f, int g)
{
   float v = f[0];
#pragma unroll
   for (int c = 1; c < 6; ++c)
      if (g == c)
         v = f[c];
   return v;
}

// lane g of a group of G stores components g, g + G, ... < 6: out = base + f
template <int G>
__device__ __forceinline__ void store6(float* __restrict__ out, const float* __restrict__ base, int s, int g,
   const float* f)
{
#pragma unroll
   for (int c0 = 0; c0 < 6; c0 += G) {
      const int c = c0 + g;
      if (c < 6) {
         float v = pick6(f, c);
         if (base)
            v += base[8 * s + c];
         out[8 * s + c] = v;
      }
   }
}

// ---------------------------------------------------------------------------
// mutual field -T u, i side (pair_ufield_v2)

__device__ __forceinline__ void ufield_i(const PairParams& P, float r2, float3 d, float uscale, float pdi, float pti,
   float pdk, float ptk, const float* uk, float* f)
{
   float invr = rsqrtf(r2);
   float r = r2 * invr;
   float rr2 = invr * invr;
   float rr3 = invr * rr2;
   float rr5 = 3.f * rr3 * rr2;
   float s3, s5, s7;
   thole_damp(r, pdi, pair_gamma(P, pti, ptk), pdk, s3, s5, s7);
   float b1, b2;
   if (P.ewald) {
      float e1, e2, e3;
      ewald_bn(P, r, invr, rr2, e1, e2, e3);
      b1 = e1 - (1.f - uscale * s3) * rr3;
      b2 = e2 - (1.f - uscale * s5) * rr5;
   } else {
      b1 = uscale * s3 * rr3;
      b2 = uscale * s5 * rr5;
   }
   float c = b2 * (d.x * uk[0] + d.y * uk[1] + d.z * uk[2]);
   f[0] += c * d.x - b1 * uk[0];
   f[1] += c * d.y - b1 * uk[1];
   f[2] += c * d.z - b1 * uk[2];
   c = b2 * (d.x * uk[3] + d.y * uk[4] + d.z * uk[5]);
   f[3] += c * d.x - b1 * uk[3];
   f[4] += c * d.y - b1 * uk[4];
   f[5] += c * d.z - b1 * uk[5];
}

// DIR: the dipoles are the CG search direction p = z + b p_old, formed
// from u8 = p_old, z8 and b (scal) as each row is read
template <int G, bool DIR>
__device__ __forceinline__ void urow(const float* __restrict__ u8, const float* __restrict__ z8, int j, float bd,
   float bp, float* v)
{
   if (DIR)
      dir_row(u8, z8, j, bd, bp, v);
   else
      load8(u8, j, v);
}

template <int G, bool DIR>
__global__ void __launch_bounds__(256) k_ufield_real(PairParams P, int npad, const int* __restrict__ nbr,
   const int* __restrict__ nnbr, const int* __restrict__ sp_start, const int* __restrict__ sp_j,
   const float4* __restrict__ sp_sc, const float4* __restrict__ spos, const float* __restrict__ u8,
   const float* __restrict__ z8, const double* __restrict__ scal, const float* __restrict__ base8,
   float* __restrict__ out8)
{
   pdl_wait();
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid / G, g = tid % G;
   if (i >= npad)
      return;
   float bd = 0.f, bp = 0.f;
   if (DIR) {
      bd = (float)scal[S_B_D];
      bp = (float)scal[S_B_P];
   }
   float f[6] = {0, 0, 0, 0, 0, 0};
   if (i < P.n) {
      const float4 pi = spos[i];  // w = pdamp
      const float pti = u8[8 * i + 6];
      const int* row = nbr + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      int k = g;
      // two neighbours per trip: both sets of loads are in flight together;
      // each neighbour is one 16-byte position and one 32-byte row
      for (; k + G < cnt; k += 2 * G) {
         const int j0 = row[k], j1 = row[k + G];
         const float4 p0 = spos[j0], p1 = spos[j1];
         float u0[8], u1[8];
         urow<G, DIR>(u8, z8, j0, bd, bp, u0);
         urow<G, DIR>(u8, z8, j1, bd, bp, u1);
         const float3 s0 = sep(P, pi, p0), s1 = sep(P, pi, p1);
         const float r0 = s0.x * s0.x + s0.y * s0.y + s0.z * s0.z;
         const float r1 = s1.x * s1.x + s1.y * s1.y + s1.z * s1.z;
         if (r0 <= P.cut2)
            ufield_i(P, r0, s0, 1.f, pi.w, pti, p0.w, u0[6], u0, f);
         if (r1 <= P.cut2)
            ufield_i(P, r1, s1, 1.f, pi.w, pti, p1.w, u1[6], u1, f);
      }
      if (k < cnt) {
         const int j = row[k];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float uk[8];
            urow<G, DIR>(u8, z8, j, bd, bp, uk);
            ufield_i(P, r2, d, 1.f, pi.w, pti, pk.w, uk[6], uk, f);
         }
      }
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G) {
         const int j = sp_j[q];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float uk[8];
            urow<G, DIR>(u8, z8, j, bd, bp, uk);
            ufield_i(P, r2, d, sp_sc[q].w, pi.w, pti, pk.w, uk[6], uk, f);
         }
      }
   }
   pdl_trigger();
   group_reduce<G, 6>(f);
   store6<G>(out8, i < P.n ? base8 : nullptr, i, g, f);
}

// ---------------------------------------------------------------------------
// permanent field, i side (pair_dfield_v2)

__device__ __forceinline__ void dfield_i(const PairParams& P, float r2, float3 d, float dscale, float pscale,
   float pdi, float pti, float pdk, float ptk, const float* mk, float* f)
{
   float invr = rsqrtf(r2);
   float r = r2 * invr;
   float rr2 = invr * invr;
   float rr3 = invr * rr2;
   float rr5 = 3.f * rr3 * rr2;
   float rr7 = 5.f * rr5 * rr2;
   float s3, s5, s7;
   thole_damp(r, pdi, pair_gamma(P, pti, ptk), pdk, s3, s5, s7);
   float e1 = 0.f, e2 = 0.f, e3 = 0.f;
   if (P.ewald)
      ewald_bn(P, r, invr, rr2, e1, e2, e3);
   // mk: c, dx, dy, dz, qxx, qyy, qzz, qxy, qxz, qyz
   const float dkr = mk[1] * d.x + mk[2] * d.y + mk[3] * d.z;
   const float qkx = mk[4] * d.x + mk[7] * d.y + mk[8] * d.z;
   const float qky = mk[7] * d.x + mk[5] * d.y + mk[9] * d.z;
   const float qkz = mk[8] * d.x + mk[9] * d.y + mk[6] * d.z;
   const float qkr = qkx * d.x + qky * d.y + qkz * d.z;
   float b1, b2, b3;
   if (P.ewald) {
      b1 = e1 - (1.f - dscale * s3) * rr3;
      b2 = e2 - (1.f - dscale * s5) * rr5;
      b3 = e3 - (1.f - dscale * s7) * rr7;
   } else {
      b1 = dscale * s3 * rr3;
      b2 = dscale * s5 * rr5;
      b3 = dscale * s7 * rr7;
   }
   float c1 = -(b1 * mk[0] - b2 * dkr + b3 * qkr);
   float fx = c1 * d.x - b1 * mk[1] + 2.f * b2 * qkx;
   float fy = c1 * d.y - b1 * mk[2] + 2.f * b2 * qky;
   float fz = c1 * d.z - b1 * mk[3] + 2.f * b2 * qkz;
   f[0] += fx;
   f[1] += fy;
   f[2] += fz;
   if (pscale != dscale) {
      if (P.ewald) {
         b1 = e1 - (1.f - pscale * s3) * rr3;
         b2 = e2 - (1.f - pscale * s5) * rr5;
         b3 = e3 - (1.f - pscale * s7) * rr7;
      } else {
         b1 = pscale * s3 * rr3;
         b2 = pscale * s5 * rr5;
         b3 = pscale * s7 * rr7;
      }
      c1 = -(b1 * mk[0] - b2 * dkr + b3 * qkr);
      fx = c1 * d.x - b1 * mk[1] + 2.f * b2 * qkx;
      fy = c1 * d.y - b1 * mk[2] + 2.f * b2 * qky;
      fz = c1 * d.z - b1 * mk[3] + 2.f * b2 * qkz;
   }
   f[3] += fx;
   f[4] += fy;
   f[5] += fz;
}

// one 48-byte multipole row: q, d xyz, qxx, qyy, qzz, qxy, qxz, qyz, thole, polarizability
__device__ __forceinline__ void load12(const float* __restrict__ rp, int s, float* m)
{
   const float4* p = reinterpret_cast<const float4*>(rp + 12 * s);
#pragma unroll
   for (int c = 0; c < 3; ++c) {
      const float4 v = p[c];
      m[4 * c] = v.x;
      m[4 * c + 1] = v.y;
      m[4 * c + 2] = v.z;
      m[4 * c + 3] = v.w;
   }
}

template <int G>
__global__ void __launch_bounds__(256) k_dfield_real(PairParams P, int npad, const int* __restrict__ nbr,
   const int* __restrict__ nnbr, const int* __restrict__ sp_start, const int* __restrict__ sp_j,
   const float4* __restrict__ sp_sc, const float4* __restrict__ spos, const float* __restrict__ rp,
   const float* __restrict__ base8, const float* __restrict__ exfld, float* __restrict__ out8)
{
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid / G, g = tid % G;
   if (i >= npad)
      return;
   float f[6] = {0, 0, 0, 0, 0, 0};
   if (i < P.n) {
      const float4 pi = spos[i];
      const float pti = rp[12 * i + 10];
      const int* row = nbr + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      for (int k = g; k < cnt; k += G) {
         const int j = row[k];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float mk[12];
            load12(rp, j, mk);
            dfield_i(P, r2, d, 1.f, 1.f, pi.w, pti, pk.w, mk[10], mk, f);
         }
      }
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G) {
         const int j = sp_j[q];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float mk[12];
            load12(rp, j, mk);
            const float4 sc = sp_sc[q];
            dfield_i(P, r2, d, sc.y, sc.z, pi.w, pti, pk.w, mk[10], mk, f);
         }
      }
   }
   group_reduce<G, 6>(f);
   if (i < P.n) {
      // uniform external field on both sets (extfieldModifyDField_cu1,
      // src/cu/amoeba/empole.cu:139-159); zero when none is set
      const float e0 = exfld[0], e1 = exfld[1], e2 = exfld[2];
      f[0] += e0;
      f[1] += e1;
      f[2] += e2;
      f[3] += e0;
      f[4] += e1;
      f[5] += e2;
   }
   store6<G>(out8, i < P.n ? base8 : nullptr, i, g, f);
}

// ---------------------------------------------------------------------------
// sparse preconditioner: z_i = udiag alpha_i r_i + sum_k alpha_i alpha_k T_ik r_k

__device__ __forceinline__ void precond_i(const PairParams& P, float r2, float3 d, float us, float poli, float pdi, float pti, float pdk,
   const float* rk, float* f)
{
   const float polk = rk[7];
   float invr = rsqrtf(r2);
   float r = r2 * invr;
   float s3, s5, s7;
   thole_damp(r, pdi, pair_gamma(P, pti, rk[6]), pdk, s3, s5, s7);
   const float polik = poli * polk;
   const float ir3 = invr * invr * invr;
   const float rr3 = us * s3 * polik * ir3;
   const float rr5 = 3.f * us * s5 * polik * ir3 * invr * invr;
   float c = rr5 * (d.x * rk[0] + d.y * rk[1] + d.z * rk[2]);
   f[0] += c * d.x - rr3 * rk[0];
   f[1] += c * d.y - rr3 * rk[1];
   f[2] += c * d.z - rr3 * rk[2];
   c = rr5 * (d.x * rk[3] + d.y * rk[4] + d.z * rk[5]);
   f[3] += c * d.x - rr3 * rk[3];
   f[4] += c * d.y - rr3 * rk[4];
   f[5] += c * d.z - rr3 * rk[5];
}

// the preconditioner row of slot i: the off-diagonal sums f[6] (reduced
// over the group); z_c = udiag alpha_i r_c + f_c
template <int G>
__device__ __forceinline__ void precond_row(const PairParams& P, int i, int g, float* f,
   const int* __restrict__ nbr, const int* __restrict__ nnbr, const int* __restrict__ sp_start,
   const int* __restrict__ sp_j, const float4* __restrict__ sp_sc, const float4* __restrict__ spos,
   const float* __restrict__ r8)
{
#pragma unroll
   for (int c = 0; c < 6; ++c)
      f[c] = 0.f;
   const float poli = r8[8 * i + 7];
   if (i < P.n) {
      const float4 pi = spos[i];
      const float pti = r8[8 * i + 6];
      const int* row = nbr + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      int k = g;
      for (; k + G < cnt; k += 2 * G) {
         const int j0 = row[k], j1 = row[k + G];
         const float4 p0 = spos[j0], p1 = spos[j1];
         float r0v[8], r1v[8];
         load8(r8, j0, r0v);
         load8(r8, j1, r1v);
         const float3 s0 = sep(P, pi, p0), s1 = sep(P, pi, p1);
         const float q0 = s0.x * s0.x + s0.y * s0.y + s0.z * s0.z;
         const float q1 = s1.x * s1.x + s1.y * s1.y + s1.z * s1.z;
         if (q0 <= P.cut2)
            precond_i(P, q0, s0, 1.f, poli, pi.w, pti, p0.w, r0v, f);
         if (q1 <= P.cut2)
            precond_i(P, q1, s1, 1.f, poli, pi.w, pti, p1.w, r1v, f);
      }
      if (k < cnt) {
         const int j = row[k];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float rk[8];
            load8(r8, j, rk);
            precond_i(P, r2, d, 1.f, poli, pi.w, pti, pk.w, rk, f);
         }
      }
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G) {
         const int j = sp_j[q];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float rk[8];
            load8(r8, j, rk);
            precond_i(P, r2, d, sp_sc[q].w, poli, pi.w, pti, pk.w, rk, f);
         }
      }
   }
   group_reduce<G, 6>(f);
}

template <int G>
__global__ void __launch_bounds__(256) k_precond_sparse(PairParams P, int npad, float udiag,
   const int* __restrict__ nbr, const int* __restrict__ nnbr, const int* __restrict__ sp_start,
   const int* __restrict__ sp_j, const float4* __restrict__ sp_sc, const float4* __restrict__ spos,
   const float* __restrict__ r8, float* __restrict__ z8)
{
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid / G, g = tid % G;
   if (i >= npad)
      return;
   float f[6];
   precond_row<G>(P, i, g, f, nbr, nnbr, sp_start, sp_j, sp_sc, spos, r8);
   const float poli = r8[8 * i + 7];
#pragma unroll
   for (int c0 = 0; c0 < 6; c0 += G) {
      const int c = c0 + g;
      if (c < 6)
         z8[8 * i + c] = udiag * poli * r8[8 * i + c] + pick6(f, c);
   }
}

// z = M r fused with the partial sums r.z, r.r (d and p) and, in the last
// block, the CG scalars.  Slots are visited block-strided, 256 / G per
// block per trip (npad is a multiple of 32, so every lane of a block makes
// the same trips); at most RED_MAX blocks.
template <int G>
__global__ void __launch_bounds__(256, 4) k_precond_sparse_dots(PairParams P, int npad, float udiag,
   const int* __restrict__ nbr, const int* __restrict__ nnbr, const int* __restrict__ sp_start,
   const int* __restrict__ sp_j, const float4* __restrict__ sp_sc, const float4* __restrict__ spos,
   const float* __restrict__ r8, float* __restrict__ z8, PcgDots D)
{
   pdl_wait();
   __shared__ double sh[64];
   constexpr int PER = 256 / G;
   const int g = threadIdx.x % G;
   float rz_d = 0.f, rz_p = 0.f, rr_d = 0.f, rr_p = 0.f;
   for (int i = blockIdx.x * PER + threadIdx.x / G; i < npad; i += gridDim.x * PER) {
      float f[6];
      precond_row<G>(P, i, g, f, nbr, nnbr, sp_start, sp_j, sp_sc, spos, r8);
      const float poli = r8[8 * i + 7];
#pragma unroll
      for (int c0 = 0; c0 < 6; c0 += G) {
         const int c = c0 + g;
         if (c < 6) {
            const float r = r8[8 * i + c];
            const float z = udiag * poli * r + pick6(f, c);
            z8[8 * i + c] = z;
            if (D.init)
               D.conj[8 * i + c] = z;
            if (c < 3) {
               rz_d += r * z;
               rr_d += r * r;
            } else {
               rz_p += r * z;
               rr_p += r * r;
            }
         }
      }
   }
   const float pv[4] = {rz_d, rz_p, rr_d, rr_p};
   pdl_trigger();
   store_partials_f<4>(D.red, R_RZ_D, pv, sh);
   if (!last_block(D.state + ST_TICKET0))
      return;
   double tot[4];
   sum_slots(D.red, R_RZ_D, 4, gridDim.x, sh, tot);
   if (threadIdx.x == 0)
      pcg_scalars(tot, D.scal, D.state, D.init, D.n, D.debye, D.poleps, D.politer, D.miniter, D.handle,
         D.use_handle);
}

// ---------------------------------------------------------------------------
// Staged field and preconditioner kernels (t9gb_pair_staging): one CTA per
// 32-slot block (32 atoms x G lanes).  The block's j-blocks (the 32-slot
// blocks its sub-list entries fall in, listed by the filter) are copied into
// shared memory by the bulk-copy engine (cp.async.bulk: one 512-byte
// position copy and one 1-KB row copy per j-block, completing on an
// mbarrier), and every neighbour row is then read from shared memory through
// the entry's local index: one coalesced 2-byte index load per neighbour
// instead of a dependent scattered 48-byte global gather.  The neighbour
// order and the arithmetic are those of the global-memory kernels, so the
// fields are bit-identical to theirs; a block with more j-blocks than
// STAGE_JB_CAP reads its rows from global memory the same way.

constexpr unsigned STAGE_POS_BYTES = 32 * 16;   // one j-block of positions
constexpr unsigned STAGE_ROW_BYTES = 32 * 32;   // one j-block of 8-float rows
constexpr size_t STAGE_SMEM = (size_t)STAGE_JB_CAP * (STAGE_POS_BYTES + STAGE_ROW_BYTES);

// Stages the j-blocks jl[0..cnt) of positions and rows and waits for them
// (phase `phase` of the CTA's mbarrier); a wait that runs out is recorded in
// *err.  The caller has synchronised the CTA since its last read of the
// staging buffers.
__device__ __forceinline__ void stage_rows(unsigned char* stg, unsigned bar, unsigned phase, const int* __restrict__ jl,
   int cnt, const float4* __restrict__ spos, const float* __restrict__ r8, int* __restrict__ err)
{
   const unsigned pos_s = (unsigned)__cvta_generic_to_shared(stg);
   const unsigned row_s = pos_s + STAGE_JB_CAP * STAGE_POS_BYTES;
   if (threadIdx.x == 0)
      mbar_expect_tx(bar, (unsigned)cnt * (STAGE_POS_BYTES + STAGE_ROW_BYTES));
   // the previous pass's reads of the buffers (generic proxy) before the
   // copies' writes (async proxy)
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   for (int q = threadIdx.x; q < cnt; q += blockDim.x) {
      const int jb = jl[q];
      bulk_g2s(pos_s + q * STAGE_POS_BYTES, spos + (size_t)jb * 32, STAGE_POS_BYTES, bar);
      bulk_g2s(row_s + q * STAGE_ROW_BYTES, r8 + (size_t)jb * 32 * 8, STAGE_ROW_BYTES, bar);
   }
   if (mbar_wait_bounded(bar, phase))
      return;
   if (threadIdx.x == 0)
      atomicExch(err, 1);
   mbar_wait_bounded(bar, phase);  // the copies in flight, before the buffers are reused
}

// neighbour row L from the staged buffers
__device__ __forceinline__ void staged_row(const unsigned char* stg, int L, float4& p, float* v)
{
   p = reinterpret_cast<const float4*>(stg)[L];
   const float4* r = reinterpret_cast<const float4*>(stg + STAGE_JB_CAP * STAGE_POS_BYTES) + 2 * L;
   const float4 x = r[0], y = r[1];
   v[0] = x.x;
   v[1] = x.y;
   v[2] = x.z;
   v[3] = x.w;
   v[4] = y.x;
   v[5] = y.y;
   v[6] = y.z;
   v[7] = y.w;
}

template <int G>
__global__ void __launch_bounds__(32 * G) k_ufield_stg(PairParams P, const int* __restrict__ nbr,
   const unsigned short* __restrict__ nbr_l, const int* __restrict__ nnbr, const int* __restrict__ jbl,
   const int* __restrict__ jbn, const int* __restrict__ sp_start, const int* __restrict__ sp_j,
   const float4* __restrict__ sp_sc, const float4* __restrict__ spos, const float* __restrict__ u8,
   const float* __restrict__ base8, float* __restrict__ out8, int* __restrict__ err)
{
   pdl_wait();
   extern __shared__ __align__(128) unsigned char stg[];
   __shared__ __align__(8) unsigned long long bar;
   const int blk = blockIdx.x;
   const int i = blk * 32 + threadIdx.x / G, g = threadIdx.x % G;
   const int nj = jbn[blk];
   const bool staged = nj <= STAGE_JB_CAP;
   if (staged) {
      const unsigned bar_s = (unsigned)__cvta_generic_to_shared(&bar);
      if (threadIdx.x == 0)
         mbar_init(bar_s, 1);
      __syncthreads();
      stage_rows(stg, bar_s, 0, jbl + (size_t)blk * STAGE_JB_CAP, nj, spos, u8, err);
   }
   float f[6] = {0, 0, 0, 0, 0, 0};
   if (i < P.n) {
      const float4 pi = spos[i];
      const float pti = u8[8 * i + 6];
      const int cnt = nnbr[i];
      int k = g;
      if (staged) {
         const unsigned short* row = nbr_l + (size_t)i * P.cap;
         for (; k + G < cnt; k += 2 * G) {
            float4 p0, p1;
            float u0[8], u1[8];
            staged_row(stg, row[k], p0, u0);
            staged_row(stg, row[k + G], p1, u1);
            const float3 s0 = sep(P, pi, p0), s1 = sep(P, pi, p1);
            const float r0 = s0.x * s0.x + s0.y * s0.y + s0.z * s0.z;
            const float r1 = s1.x * s1.x + s1.y * s1.y + s1.z * s1.z;
            if (r0 <= P.cut2)
               ufield_i(P, r0, s0, 1.f, pi.w, pti, p0.w, u0[6], u0, f);
            if (r1 <= P.cut2)
               ufield_i(P, r1, s1, 1.f, pi.w, pti, p1.w, u1[6], u1, f);
         }
         if (k < cnt) {
            float4 pk;
            float uk[8];
            staged_row(stg, row[k], pk, uk);
            const float3 d = sep(P, pi, pk);
            const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
            if (r2 <= P.cut2)
               ufield_i(P, r2, d, 1.f, pi.w, pti, pk.w, uk[6], uk, f);
         }
      } else {
         const int* row = nbr + (size_t)i * P.cap;
         for (; k + G < cnt; k += 2 * G) {
            const int j0 = row[k], j1 = row[k + G];
            const float4 p0 = spos[j0], p1 = spos[j1];
            float u0[8], u1[8];
            load8(u8, j0, u0);
            load8(u8, j1, u1);
            const float3 s0 = sep(P, pi, p0), s1 = sep(P, pi, p1);
            const float r0 = s0.x * s0.x + s0.y * s0.y + s0.z * s0.z;
            const float r1 = s1.x * s1.x + s1.y * s1.y + s1.z * s1.z;
            if (r0 <= P.cut2)
               ufield_i(P, r0, s0, 1.f, pi.w, pti, p0.w, u0[6], u0, f);
            if (r1 <= P.cut2)
               ufield_i(P, r1, s1, 1.f, pi.w, pti, p1.w, u1[6], u1, f);
         }
         if (k < cnt) {
            const int j = row[k];
            const float4 pk = spos[j];
            const float3 d = sep(P, pi, pk);
            const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
            if (r2 <= P.cut2) {
               float uk[8];
               load8(u8, j, uk);
               ufield_i(P, r2, d, 1.f, pi.w, pti, pk.w, uk[6], uk, f);
            }
         }
      }
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G) {
         const int j = sp_j[q];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float uk[8];
            load8(u8, j, uk);
            ufield_i(P, r2, d, sp_sc[q].w, pi.w, pti, pk.w, uk[6], uk, f);
         }
      }
   }
   pdl_trigger();
   group_reduce<G, 6>(f);
   store6<G>(out8, i < P.n ? base8 : nullptr, i, g, f);
}

// the preconditioner row of slot i, rows from the staged buffers
template <int G>
__device__ __forceinline__ void precond_row_stg(const PairParams& P, int i, int g, const unsigned char* stg, float* f,
   const unsigned short* __restrict__ nbr_l, const int* __restrict__ nnbr, const int* __restrict__ sp_start,
   const int* __restrict__ sp_j, const float4* __restrict__ sp_sc, const float4* __restrict__ spos,
   const float* __restrict__ r8)
{
#pragma unroll
   for (int c = 0; c < 6; ++c)
      f[c] = 0.f;
   const float poli = r8[8 * i + 7];
   if (i < P.n) {
      const float4 pi = spos[i];
      const float pti = r8[8 * i + 6];
      const unsigned short* row = nbr_l + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      int k = g;
      for (; k + G < cnt; k += 2 * G) {
         float4 p0, p1;
         float r0v[8], r1v[8];
         staged_row(stg, row[k], p0, r0v);
         staged_row(stg, row[k + G], p1, r1v);
         const float3 s0 = sep(P, pi, p0), s1 = sep(P, pi, p1);
         const float q0 = s0.x * s0.x + s0.y * s0.y + s0.z * s0.z;
         const float q1 = s1.x * s1.x + s1.y * s1.y + s1.z * s1.z;
         if (q0 <= P.cut2)
            precond_i(P, q0, s0, 1.f, poli, pi.w, pti, p0.w, r0v, f);
         if (q1 <= P.cut2)
            precond_i(P, q1, s1, 1.f, poli, pi.w, pti, p1.w, r1v, f);
      }
      if (k < cnt) {
         float4 pk;
         float rk[8];
         staged_row(stg, row[k], pk, rk);
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2)
            precond_i(P, r2, d, 1.f, poli, pi.w, pti, pk.w, rk, f);
      }
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G) {
         const int j = sp_j[q];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float rk[8];
            load8(r8, j, rk);
            precond_i(P, r2, d, sp_sc[q].w, poli, pi.w, pti, pk.w, rk, f);
         }
      }
   }
   group_reduce<G, 6>(f);
}

// z = M r with the r.z / r.r partial sums and, in the last block, the CG
// scalars (k_precond_sparse_dots), one 32-slot block per CTA pass; a CTA
// takes blocks blockIdx.x, + gridDim.x, ... (at most RED_MAX CTAs), the
// staging mbarrier's phase flipping with each staged pass.
template <int G>
__global__ void __launch_bounds__(32 * G) k_precond_dots_stg(PairParams P, int nblk, float udiag,
   const int* __restrict__ nbr, const unsigned short* __restrict__ nbr_l, const int* __restrict__ nnbr,
   const int* __restrict__ jbl, const int* __restrict__ jbn, const int* __restrict__ sp_start,
   const int* __restrict__ sp_j, const float4* __restrict__ sp_sc, const float4* __restrict__ spos,
   const float* __restrict__ r8, float* __restrict__ z8, PcgDots D, int* __restrict__ err)
{
   pdl_wait();
   extern __shared__ __align__(128) unsigned char stg[];
   __shared__ __align__(8) unsigned long long bar;
   __shared__ double sh[64];
   const unsigned bar_s = (unsigned)__cvta_generic_to_shared(&bar);
   if (threadIdx.x == 0)
      mbar_init(bar_s, 1);
   __syncthreads();
   const int g = threadIdx.x % G;
   float rz_d = 0.f, rz_p = 0.f, rr_d = 0.f, rr_p = 0.f;
   unsigned phase = 0;
   for (int blk = blockIdx.x; blk < nblk; blk += gridDim.x) {
      const int i = blk * 32 + threadIdx.x / G;
      const int nj = jbn[blk];
      float f[6];
      if (nj <= STAGE_JB_CAP) {
         __syncthreads();  // the previous pass has read the buffers
         stage_rows(stg, bar_s, phase, jbl + (size_t)blk * STAGE_JB_CAP, nj, spos, r8, err);
         phase ^= 1u;
         precond_row_stg<G>(P, i, g, stg, f, nbr_l, nnbr, sp_start, sp_j, sp_sc, spos, r8);
      } else {
         precond_row<G>(P, i, g, f, nbr, nnbr, sp_start, sp_j, sp_sc, spos, r8);
      }
      const float poli = r8[8 * i + 7];
#pragma unroll
      for (int c0 = 0; c0 < 6; c0 += G) {
         const int c = c0 + g;
         if (c < 6) {
            const float r = r8[8 * i + c];
            const float z = udiag * poli * r + pick6(f, c);
            z8[8 * i + c] = z;
            if (D.init)
               D.conj[8 * i + c] = z;
            if (c < 3) {
               rz_d += r * z;
               rr_d += r * r;
            } else {
               rz_p += r * z;
               rr_p += r * r;
            }
         }
      }
   }
   const float pv[4] = {rz_d, rz_p, rr_d, rr_p};
   pdl_trigger();
   store_partials_f<4>(D.red, R_RZ_D, pv, sh);
   if (!last_block(D.state + ST_TICKET0))
      return;
   double tot[4];
   sum_slots_bd(D.red, R_RZ_D, 4, gridDim.x, sh, tot);
   if (threadIdx.x == 0)
      pcg_scalars(tot, D.scal, D.state, D.init, D.n, D.debye, D.poleps, D.politer, D.miniter, D.handle,
         D.use_handle);
}

// ---------------------------------------------------------------------------
// permanent-multipole energy, real space (pair_mpole energy terms,
// include/seq/pair_mpole.h:62-152); exclusion correction (m - 1) x bare pair
// as the reference's exclusion loop does (src/cu/amoeba/empole_cu1.cc:110)

__device__ __forceinline__ float mpole_pair_e(const float* bn, float3 d, const float* mi, const float* mk)
{
   const float dir = mi[1] * d.x + mi[2] * d.y + mi[3] * d.z;
   const float qix = mi[4] * d.x + mi[7] * d.y + mi[8] * d.z;
   const float qiy = mi[7] * d.x + mi[5] * d.y + mi[9] * d.z;
   const float qiz = mi[8] * d.x + mi[9] * d.y + mi[6] * d.z;
   const float qir = qix * d.x + qiy * d.y + qiz * d.z;
   const float dkr = mk[1] * d.x + mk[2] * d.y + mk[3] * d.z;
   const float qkx = mk[4] * d.x + mk[7] * d.y + mk[8] * d.z;
   const float qky = mk[7] * d.x + mk[5] * d.y + mk[9] * d.z;
   const float qkz = mk[8] * d.x + mk[9] * d.y + mk[6] * d.z;
   const float qkr = qkx * d.x + qky * d.y + qkz * d.z;
   const float dik = mi[1] * mk[1] + mi[2] * mk[2] + mi[3] * mk[3];
   const float qik = qix * qkx + qiy * qky + qiz * qkz;
   const float diqk = mi[1] * qkx + mi[2] * qky + mi[3] * qkz;
   const float dkqi = mk[1] * qix + mk[2] * qiy + mk[3] * qiz;
   const float qiqk = 2.f * (mi[7] * mk[7] + mi[8] * mk[8] + mi[9] * mk[9]) + mi[4] * mk[4] + mi[5] * mk[5]
      + mi[6] * mk[6];
   const float t1 = mi[0] * mk[0];
   const float t2 = mk[0] * dir - mi[0] * dkr + dik;
   const float t3 = mi[0] * qkr + mk[0] * qir - dir * dkr + 2.f * (dkqi - diqk + qiqk);
   const float t4 = dir * qkr - dkr * qir - 4.f * qik;
   const float t5 = qir * qkr;
   return t1 * bn[0] + t2 * bn[1] + t3 * bn[2] + t4 * bn[3] + t5 * bn[4];
}

__device__ __forceinline__ void bare_bn5(float f, float invr, float* bn)
{
   const float rr2 = invr * invr;
   bn[0] = f * invr;
   bn[1] = bn[0] * rr2;
   bn[2] = 3.f * bn[1] * rr2;
   bn[3] = 5.f * bn[2] * rr2;
   bn[4] = 7.f * bn[3] * rr2;
}

__device__ __forceinline__ void ewald_bn5(const PairParams& P, float f, float r, float invr, float* bn)
{
   const float rr2 = invr * invr;
   const float ralpha = P.aewald * r;
   const float exp2a = __expf(-ralpha * ralpha);
   float b0 = erfc_hastings(ralpha, exp2a) * invr;
   float b1 = (b0 + P.ec1 * exp2a) * rr2;
   float b2 = (3.f * b1 + P.ec2 * exp2a) * rr2;
   float b3 = (5.f * b2 + P.ec3 * exp2a) * rr2;
   float b4 = (7.f * b3 + P.ec4 * exp2a) * rr2;
   bn[0] = f * b0;
   bn[1] = f * b1;
   bn[2] = f * b2;
   bn[3] = f * b3;
   bn[4] = f * b4;
}

// e_atom[i] = 1/2 sum over i's list and scaled partners (every pair is seen
// from both atoms); FP64 accumulation of FP32 pair energies
template <int G>
__global__ void __launch_bounds__(256) k_empole_real(PairParams P, int npad, float f, const int* __restrict__ nbr,
   const int* __restrict__ nnbr, const int* __restrict__ sp_start, const int* __restrict__ sp_j,
   const float4* __restrict__ sp_sc, const float4* __restrict__ spos, const float* __restrict__ rp,
   double* __restrict__ e_atom)
{
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid / G, g = tid % G;
   if (i >= npad)
      return;
   double e = 0;
   if (i < P.n) {
      const float4 pi = spos[i];
      float mi[12];
      load12(rp, i, mi);
      const int* row = nbr + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      for (int k = g; k < cnt; k += G) {
         const int j = row[k];
         const float3 d = sep(P, pi, spos[j]);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float mk[12], bn[5];
            load12(rp, j, mk);
            const float invr = rsqrtf(r2);
            if (P.ewald)
               ewald_bn5(P, f, r2 * invr, invr, bn);
            else
               bare_bn5(f, invr, bn);
            e += (double)mpole_pair_e(bn, d, mi, mk);
         }
      }
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G) {
         const int j = sp_j[q];
         const float3 d = sep(P, pi, spos[j]);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            float mk[12], bn[5];
            load12(rp, j, mk);
            const float invr = rsqrtf(r2);
            const float ms = sp_sc[q].x;
            bare_bn5(f, invr, bn);
            float eb = mpole_pair_e(bn, d, mi, mk);
            if (P.ewald) {
               ewald_bn5(P, f, r2 * invr, invr, bn);
               e += (double)mpole_pair_e(bn, d, mi, mk) + (double)(ms - 1.f) * eb;
            } else {
               e += (double)(ms * eb);
            }
         }
      }
   }
#pragma unroll
   for (int o = G / 2; o > 0; o >>= 1)
      e += __shfl_xor_sync(0xffffffffu, e, o);
   if (g == 0)
      e_atom[i] = i < P.n ? 0.5 * e : 0.0;
}

// ---------------------------------------------------------------------------
// launchers


static constexpr int PAIR_THREADS = 256;

// ---------------------------------------------------------------------------
// Per-step sub-lists: one CTA per 32-slot block, warp w filtering the row of
// slot 32 b + w.  Each row of the (reused, buffered) list is filtered into
// the pairs within the cutoff and those within the preconditioner cutoff, in
// the row's order (ballot compaction), so the field and preconditioner
// kernels visit only pairs they use; the kernels repeat the same r^2 test
// with the same arithmetic.  STAGE: the block also records which 32-slot
// j-blocks its entries fall in (a bitmap over all blocks in shared memory),
// lists them in ascending order, and rewrites every entry as a local index
// into that list (position x 32 + slot within the j-block), which is where
// the staged kernels find the row in shared memory.
template <bool STAGE>
__global__ void __launch_bounds__(1024) k_list_filter(PairParams P, float cutp2, int npad, const int* __restrict__ nbr,
   const int* __restrict__ nnbr, const float4* __restrict__ spos, int* __restrict__ nbrc, int* __restrict__ nnbrc,
   int* __restrict__ nbrp, int* __restrict__ nnbrp, int* __restrict__ jbl, int* __restrict__ jbn,
   unsigned short* __restrict__ nbrc_l, unsigned short* __restrict__ nbrp_l)
{
   extern __shared__ unsigned bits_sm[];
   __shared__ int total_sm;
   const int words = (npad / 32 + 31) / 32;
   unsigned* bm = bits_sm;
   int* pre = reinterpret_cast<int*>(bits_sm + words);
   if (STAGE) {
      for (int w = threadIdx.x; w < words; w += blockDim.x)
         bm[w] = 0u;
      __syncthreads();
   }
   const int blk = blockIdx.x;
   const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
   const int i = blk * 32 + warp;
   int oc = 0, op = 0;
   if (i < P.n) {
      const float4 pi = spos[i];
      const int* row = nbr + (size_t)i * P.cap;
      int* rc = nbrc + (size_t)i * P.cap;
      int* rp = nbrp + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      const unsigned lt = (1u << lane) - 1u;
      for (int k0 = 0; k0 < cnt; k0 += 32) {
         const int k = k0 + lane;
         bool inc = false, inp = false;
         int j = 0;
         if (k < cnt) {
            j = row[k];
            const float3 d = sep(P, pi, spos[j]);
            const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
            inc = r2 <= P.cut2;
            inp = r2 <= cutp2;
         }
         const unsigned mc = __ballot_sync(0xffffffffu, inc), mp = __ballot_sync(0xffffffffu, inp);
         if (inc)
            rc[oc + __popc(mc & lt)] = j;
         if (inp)
            rp[op + __popc(mp & lt)] = j;
         if (STAGE && (inc || inp))
            atomicOr(&bm[j >> 10], 1u << ((j >> 5) & 31));
         oc += __popc(mc);
         op += __popc(mp);
      }
   }
   if (lane == 0) {
      nnbrc[i] = oc;
      nnbrp[i] = op;
   }
   if (!STAGE)
      return;
   __syncthreads();
   // set bits before each word, and the block's j-block list
   if (warp == 0) {
      int run = 0;
      for (int w0 = 0; w0 < words; w0 += 32) {
         const int w = w0 + lane;
         const int c = w < words ? __popc(bm[w]) : 0;
         int incl = c;
#pragma unroll
         for (int o = 1; o < 32; o <<= 1) {
            const int t = __shfl_up_sync(0xffffffffu, incl, o);
            if (lane >= o)
               incl += t;
         }
         if (w < words)
            pre[w] = run + incl - c;
         run += __shfl_sync(0xffffffffu, incl, 31);
      }
      if (lane == 0) {
         total_sm = run;
         jbn[blk] = run;
      }
   }
   __syncthreads();
   const int total = total_sm;
   if (total > STAGE_JB_CAP)
      return;  // this block reads its rows from global memory
   for (int w = threadIdx.x; w < words; w += blockDim.x) {
      unsigned m = bm[w];
      int q = pre[w];
      while (m) {
         const int b = __ffs(m) - 1;
         jbl[(size_t)blk * STAGE_JB_CAP + q] = w * 32 + b;
         ++q;
         m &= m - 1u;
      }
   }
   if (i < P.n) {
      const int* rc = nbrc + (size_t)i * P.cap;
      const int* rp = nbrp + (size_t)i * P.cap;
      unsigned short* lc = nbrc_l + (size_t)i * P.cap;
      unsigned short* lp = nbrp_l + (size_t)i * P.cap;
      for (int k = lane; k < oc; k += 32) {
         const int j = rc[k], jb = j >> 5;
         const int q = pre[jb >> 5] + __popc(bm[jb >> 5] & ((1u << (jb & 31)) - 1u));
         lc[k] = (unsigned short)(q * 32 + (j & 31));
      }
      for (int k = lane; k < op; k += 32) {
         const int j = rp[k], jb = j >> 5;
         const int q = pre[jb >> 5] + __popc(bm[jb >> 5] & ((1u << (jb & 31)) - 1u));
         lp[k] = (unsigned short)(q * 32 + (j & 31));
      }
   }
}

int launch_list_filter(Context* ctx)
{
   PairParams P = make_params(ctx, ctx->cfg.cutoff);
   const double cp = ctx->cfg.usolve_cutoff + ctx->cfg.pbuffer;
   const float cutp2 = cp * cp > 3.0e38 ? 3.0e38f : (float)(cp * cp);
   const int nblk = ctx->npad / 32;
   const int words = (nblk + 31) / 32;
   const size_t smem = sizeof(unsigned) * 2 * (size_t)words;
   if (ctx->pair_staged)
      k_list_filter<true><<<nblk, 1024, smem, ctx->stream>>>(P, cutp2, ctx->npad, ctx->nbr, ctx->nnbr, ctx->spos,
         ctx->nbrc, ctx->nnbrc, ctx->nbrp, ctx->nnbrp, ctx->jbl, ctx->jbn, ctx->nbrc_l, ctx->nbrp_l);
   else
      k_list_filter<false><<<nblk, 1024, 0, ctx->stream>>>(P, cutp2, ctx->npad, ctx->nbr, ctx->nnbr, ctx->spos,
         ctx->nbrc, ctx->nnbrc, ctx->nbrp, ctx->nnbrp, ctx->jbl, ctx->jbn, ctx->nbrc_l, ctx->nbrp_l);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// lanes per atom of the three field kernels (8, 16 or 32; t9gb_pair_lanes)
#define T9_LANES_DISPATCH(KERNEL, ...)                                                                                 \
   do {                                                                                                                \
      const int g_ = ctx->pair_lanes;                                                                                  \
      const int nb_ = grid_for((long long)ctx->npad * g_, PAIR_THREADS);                                               \
      if (g_ == 4)                                                                                                     \
         KERNEL<4><<<nb_, PAIR_THREADS, 0, ctx->stream>>>(__VA_ARGS__);                                                \
      else if (g_ == 8)                                                                                                \
         KERNEL<8><<<nb_, PAIR_THREADS, 0, ctx->stream>>>(__VA_ARGS__);                                                \
      else if (g_ == 32)                                                                                               \
         KERNEL<32><<<nb_, PAIR_THREADS, 0, ctx->stream>>>(__VA_ARGS__);                                               \
      else                                                                                                             \
         KERNEL<16><<<nb_, PAIR_THREADS, 0, ctx->stream>>>(__VA_ARGS__);                                               \
   } while (0)

// the same for kernels with a second template parameter
#define T9_LANES_DISPATCH2(KERNEL, ARG, ...)                                                                           \
   do {                                                                                                                \
      const int g_ = ctx->pair_lanes;                                                                                  \
      const int nb_ = grid_for((long long)ctx->npad * g_, PAIR_THREADS);                                               \
      if (g_ == 4)                                                                                                     \
         KERNEL<4, ARG><<<nb_, PAIR_THREADS, 0, ctx->stream>>>(__VA_ARGS__);                                           \
      else if (g_ == 8)                                                                                                \
         KERNEL<8, ARG><<<nb_, PAIR_THREADS, 0, ctx->stream>>>(__VA_ARGS__);                                           \
      else if (g_ == 32)                                                                                               \
         KERNEL<32, ARG><<<nb_, PAIR_THREADS, 0, ctx->stream>>>(__VA_ARGS__);                                          \
      else                                                                                                             \
         KERNEL<16, ARG><<<nb_, PAIR_THREADS, 0, ctx->stream>>>(__VA_ARGS__);                                          \
   } while (0)

// the staged kernels: 4 or 8 lanes per atom
static bool staged_lanes(const Context* ctx)
{
   return ctx->pair_staged && (ctx->pair_lanes == 4 || ctx->pair_lanes == 8);
}

int pair_staging_setup()
{
   const int bytes = (int)STAGE_SMEM;
   if (cudaFuncSetAttribute(k_ufield_stg<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess ||
      cudaFuncSetAttribute(k_ufield_stg<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess ||
      cudaFuncSetAttribute(k_precond_dots_stg<4>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) !=
         cudaSuccess ||
      cudaFuncSetAttribute(k_precond_dots_stg<8>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes) != cudaSuccess)
      return T9GB_CUDA_ERR;
   return T9GB_OK;
}

int launch_ufield_real(Context* ctx, const float* u6, const float* base6, float* out6)
{
   PairParams P = make_params(ctx, ctx->cfg.cutoff);
   prof_begin(ctx, P_UFIELD_REAL);
   if (staged_lanes(ctx)) {
      auto k = ctx->pair_lanes == 8 ? k_ufield_stg<8> : k_ufield_stg<4>;
      T9_CUDA(launch_k(use_pdl(ctx), k, ctx->npad / 32, 32 * ctx->pair_lanes, STAGE_SMEM, ctx->stream, P, ctx->nbrc,
         ctx->nbrc_l, ctx->nnbrc, ctx->jbl, ctx->jbn, ctx->sp_start, ctx->sp_j, ctx->sp_sc, ctx->spos, u6, base6, out6,
         ctx->copy_err));
      prof_end(ctx);
      return T9GB_OK;
   }
   const int g = ctx->pair_lanes;
   const int nb = grid_for((long long)ctx->npad * g, PAIR_THREADS);
   auto k = g == 4 ? k_ufield_real<4, false> : g == 8 ? k_ufield_real<8, false> : g == 32 ? k_ufield_real<32, false>
                                                                                    : k_ufield_real<16, false>;
   T9_CUDA(launch_k(use_pdl(ctx), k, nb, PAIR_THREADS, 0, ctx->stream, P, ctx->npad, ctx->nbrc, ctx->nnbrc,
      ctx->sp_start, ctx->sp_j, ctx->sp_sc, ctx->spos, u6, nullptr, nullptr, base6, out6));
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int launch_ufield_real_dir(Context* ctx, const float* p6, const float* z6, const double* scal, float* out6)
{
   PairParams P = make_params(ctx, ctx->cfg.cutoff);
   prof_begin(ctx, P_UFIELD_REAL);
   T9_LANES_DISPATCH2(k_ufield_real, true, P, ctx->npad, ctx->nbrc, ctx->nnbrc, ctx->sp_start, ctx->sp_j, ctx->sp_sc,
      ctx->spos, p6, z6, scal, nullptr, out6);
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int launch_dfield_real(Context* ctx, const float* base6, float* out6)
{
   PairParams P = make_params(ctx, ctx->cfg.cutoff);
   prof_begin(ctx, P_DFIELD_REAL);
   T9_LANES_DISPATCH(k_dfield_real, P, ctx->npad, ctx->nbrc, ctx->nnbrc, ctx->sp_start, ctx->sp_j, ctx->sp_sc, ctx->spos,
      ctx->srpole, base6, ctx->exfld, out6);
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int launch_precond_sparse_dots(Context* ctx, const float* r6, float* z6, const PcgDots& D)
{
   PairParams P = make_params(ctx, ctx->cfg.usolve_cutoff + ctx->cfg.pbuffer);
   P.ewald = 0;
   const int g = ctx->pair_lanes;
   const int per = PAIR_THREADS / g;
   const int nb = std::min(RED_MAX, (ctx->npad + per - 1) / per);
   prof_begin(ctx, P_PRECOND);
   if (staged_lanes(ctx)) {
      const int nblk = ctx->npad / 32;
      auto ks = g == 8 ? k_precond_dots_stg<8> : k_precond_dots_stg<4>;
      T9_CUDA(launch_k(use_pdl(ctx), ks, std::min(RED_MAX, nblk), 32 * g, STAGE_SMEM, ctx->stream, P, nblk,
         (float)ctx->cfg.udiag, ctx->nbrp, ctx->nbrp_l, ctx->nnbrp, ctx->jbl, ctx->jbn, ctx->sp_start, ctx->sp_j,
         ctx->sp_sc, ctx->spos, r6, z6, D, ctx->copy_err));
      prof_end(ctx);
      return T9GB_OK;
   }
   auto k = g == 4 ? k_precond_sparse_dots<4> : g == 8 ? k_precond_sparse_dots<8> : g == 32
         ? k_precond_sparse_dots<32> : k_precond_sparse_dots<16>;
   T9_CUDA(launch_k(use_pdl(ctx), k, nb, PAIR_THREADS, 0, ctx->stream, P, ctx->npad, (float)ctx->cfg.udiag, ctx->nbrp,
      ctx->nnbrp, ctx->sp_start, ctx->sp_j, ctx->sp_sc, ctx->spos, r6, z6, D));
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int launch_precond_sparse(Context* ctx, const float* r6, float* z6)
{
   PairParams P = make_params(ctx, ctx->cfg.usolve_cutoff + ctx->cfg.pbuffer);
   P.ewald = 0;
   prof_begin(ctx, P_PRECOND);
   T9_LANES_DISPATCH(k_precond_sparse, P, ctx->npad, (float)ctx->cfg.udiag, ctx->nbrp, ctx->nnbrp, ctx->sp_start,
      ctx->sp_j, ctx->sp_sc, ctx->spos, r6, z6);
   prof_end(ctx);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

}  // namespace t9gb

namespace t9gb {
int launch_empole_real(Context* ctx, double* e_atom)
{
   PairParams P = make_params(ctx, ctx->cfg.cutoff);
   k_empole_real<GROUP><<<grid_for((long long)ctx->npad * GROUP, PAIR_THREADS), PAIR_THREADS, 0, ctx->stream>>>(P,
      ctx->npad, (float)ctx->cfg.electric, ctx->nbrc, ctx->nnbrc, ctx->sp_start, ctx->sp_j, ctx->sp_sc, ctx->spos,
      ctx->srpole, e_atom);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}
}  // namespace t9gb

// ---------------------------------------------------------------------------
// Descriptors of the learned initial guess.  Per slot i two rows of 32
// features, row i for the d dipoles and row npad + i for the p dipoles; every
// vector is expressed in the atom's local multipole frame (rows of
// sframe[9]), so the features are invariant under rotations of the system:
//   0-2   direct field E (d or p)
//   3     polarizability alpha_i
//   4-10  sum_k fc(r) g(r; mu, 0.5), mu = 1, 1.83, ..., 6            (count)
//   11-14 sum_k q_k fc g(r; mu, 0.75), mu = 1.5, 3, 4.5, 6           (charge)
//   15-20 sum_k q_k fc g(r; mu, 1) r_hat, mu = 2, 4.5 (x, y, z each)  (charge
//         direction)
//   21-25 sum_k alpha_k fc g(r; mu, 0.6), mu = 1, 2.25, ..., 6     (polarizability)
//   26-31 first-order mutual field of the neighbours' direct dipoles,
//         sum_k -T_ik^Thole (alpha_k E_k) * u-scale, split r < 3.5 / r >= 3.5
// over all partners within 6 A; fc = (1 + cos(pi r / 6)) / 2.
// g(r; mu, s) = exp(-(r - mu)^2 / (2 s^2)).

namespace t9gb {

constexpr float DESC_CUT = 6.f;
constexpr int NFEAT = 32;

__device__ __forceinline__ float gauss(float r, float mu, float inv2s2)
{
   const float t = r - mu;
   return __expf(-t * t * inv2s2);
}

// acc[j] += w g(r; mu0 + j dmu, s), j < N, c = 1 / (2 s^2), by the product
// recurrence g_{j+1} = g_j R_j, R_j = exp(c (2 dmu (r - mu0) - dmu^2))
// exp(-2 c dmu^2)^j: two exponentials per series instead of N (relative
// error a few units of 1e-7 over the series)
template <int N>
__device__ __forceinline__ void gauss_series(float r, float mu0, float dmu, float c, float w, float* acc)
{
   const float t = r - mu0;
   float g = __expf(-t * t * c);
   float R = __expf(c * (2.f * dmu * t - dmu * dmu));
   const float B = __expf(-2.f * c * dmu * dmu);  // constant: folded by the compiler
#pragma unroll
   for (int j = 0; j < N; ++j) {
      acc[j] += w * g;
      g *= R;
      R *= B;
   }
}

// acc layout: gr[0..7) gq[7..11) dq[11..17) ga[17..22) fd[22..28) fp[28..34)
constexpr int DACC = 34;

__device__ __forceinline__ void desc_pair(const PairParams& P, float r2, float3 d, float us, float pdi, float pti, float pdk,
   const float* uk, float qk, float* acc)
{
   const float invr = rsqrtf(r2);
   const float r = r2 * invr;
   const float fc = 0.5f * (__cosf(3.14159265f / DESC_CUT * r) + 1.f);
   gauss_series<7>(r, 1.f, 5.f / 6.f, 2.f, fc, acc);
   gauss_series<4>(r, 1.5f, 1.5f, 1.f / (2.f * 0.75f * 0.75f), qk * fc, acc + 7);
   const float h0 = qk * fc * gauss(r, 2.f, 0.5f) * invr, h1 = qk * fc * gauss(r, 4.5f, 0.5f) * invr;
   acc[11] += h0 * d.x;
   acc[12] += h0 * d.y;
   acc[13] += h0 * d.z;
   acc[14] += h1 * d.x;
   acc[15] += h1 * d.y;
   acc[16] += h1 * d.z;
   gauss_series<5>(r, 1.f, 1.25f, 1.f / (2.f * 0.6f * 0.6f), uk[7] * fc, acc + 17);
   float s3, s5, s7;
   thole_damp(r, pdi, pair_gamma(P, pti, uk[6]), pdk, s3, s5, s7);
   const float ir3 = invr * invr * invr;
   const float rr3 = us * s3 * ir3;
   const float rr5 = 3.f * us * s5 * ir3 * invr * invr;
   const float cd = rr5 * (d.x * uk[0] + d.y * uk[1] + d.z * uk[2]);
   const float cp = rr5 * (d.x * uk[3] + d.y * uk[4] + d.z * uk[5]);
   // constant indices in both branches keep acc in registers
   if (r < 3.5f) {
      acc[22] += cd * d.x - rr3 * uk[0];
      acc[23] += cd * d.y - rr3 * uk[1];
      acc[24] += cd * d.z - rr3 * uk[2];
      acc[28] += cp * d.x - rr3 * uk[3];
      acc[29] += cp * d.y - rr3 * uk[4];
      acc[30] += cp * d.z - rr3 * uk[5];
   } else {
      acc[25] += cd * d.x - rr3 * uk[0];
      acc[26] += cd * d.y - rr3 * uk[1];
      acc[27] += cd * d.z - rr3 * uk[2];
      acc[31] += cp * d.x - rr3 * uk[3];
      acc[32] += cp * d.y - rr3 * uk[4];
      acc[33] += cp * d.z - rr3 * uk[5];
   }
}

__device__ __forceinline__ void to_local(const float* F, const float* v, float* out)
{
#pragma unroll
   for (int a = 0; a < 3; ++a)
      out[a] = F[3 * a] * v[0] + F[3 * a + 1] * v[1] + F[3 * a + 2] * v[2];
}

template <int G>
__global__ void __launch_bounds__(256) k_learn_features(PairParams P, int npad, const int* __restrict__ nbr,
   const int* __restrict__ nnbr, const int* __restrict__ sp_start, const int* __restrict__ sp_j,
   const float4* __restrict__ sp_sc, const float4* __restrict__ spos, const float* __restrict__ srpole,
   const float* __restrict__ sframe, const float* __restrict__ e8, const float* __restrict__ u8,
   float* __restrict__ xf, const float* __restrict__ polar, const float* __restrict__ fstat,
   const int* __restrict__ state, __nv_bfloat16* __restrict__ xn)
{
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid / G, g = tid % G;
   if (i >= npad)
      return;
   // with the column statistics fixed (bit 0), also the BF16 network input
   const bool norm = (state[ST_LREADY] & 1) != 0;
   float acc[DACC];
#pragma unroll
   for (int c = 0; c < DACC; ++c)
      acc[c] = 0.f;
   if (i < P.n) {
      const float4 pi = spos[i];
      const float pti = u8[8 * i + 6];
      const int* row = nbr + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      for (int k = g; k < cnt; k += G) {
         const int j = row[k];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 < DESC_CUT * DESC_CUT) {
            float uk[8];
            load8(u8, j, uk);
            desc_pair(P, r2, d, 1.f, pi.w, pti, pk.w, uk, srpole[12 * j], acc);
         }
      }
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G) {
         const int j = sp_j[q];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 < DESC_CUT * DESC_CUT) {
            float uk[8];
            load8(u8, j, uk);
            desc_pair(P, r2, d, sp_sc[q].w, pi.w, pti, pk.w, uk, srpole[12 * j], acc);
         }
      }
   }
   group_reduce<G, DACC>(acc);
   if (g >= 2)
      return;
   // lane 0 writes the d row, lane 1 the p row
   const size_t row = (size_t)(g == 0 ? i : npad + i);
   float x[NFEAT];
#pragma unroll
   for (int c = 0; c < NFEAT; ++c)
      x[c] = 0.f;
   if (i < P.n) {
      float F[9];
#pragma unroll
      for (int c = 0; c < 9; ++c)
         F[c] = sframe[9 * i + c];
      float v[3];
#pragma unroll
      for (int c = 0; c < 3; ++c)
         v[c] = e8[8 * i + 3 * g + c];
      to_local(F, v, x);
      x[3] = u8[8 * i + 7];
#pragma unroll
      for (int c = 0; c < 7; ++c)
         x[4 + c] = acc[c];
#pragma unroll
      for (int c = 0; c < 4; ++c)
         x[11 + c] = acc[7 + c];
      to_local(F, acc + 11, x + 15);
      to_local(F, acc + 14, x + 18);
#pragma unroll
      for (int c = 0; c < 5; ++c)
         x[21 + c] = acc[17 + c];
      float f[6];
#pragma unroll
      for (int c = 0; c < 6; ++c)
         f[c] = g == 0 ? acc[22 + c] : acc[28 + c];
      to_local(F, f, x + 26);
      to_local(F, f + 3, x + 29);
   }
   float4* xo = reinterpret_cast<float4*>(xf + row * NFEAT);
#pragma unroll
   for (int c = 0; c < NFEAT; c += 4)
      xo[c / 4] = make_float4(x[c], x[c + 1], x[c + 2], x[c + 3]);
   if (norm) {  // as k_normalize: (x - mean) / std, zero rows where alpha = 0
      const bool live = polar[i] != 0.f;
      uint4* q = reinterpret_cast<uint4*>(xn + row * NFEAT);
#pragma unroll
      for (int c = 0; c < NFEAT; c += 8) {
         unsigned wv[4];
#pragma unroll
         for (int k = 0; k < 4; ++k) {
            const int a = c + 2 * k;
            const float v0 = live ? (x[a] - fstat[a]) * fstat[32 + a] : 0.f;
            const float v1 = live ? (x[a + 1] - fstat[a + 1]) * fstat[32 + a + 1] : 0.f;
            const __nv_bfloat162 b = __floats2bfloat162_rn(v0, v1);
            wv[k] = *reinterpret_cast<const unsigned*>(&b);
         }
         q[c / 8] = make_uint4(wv[0], wv[1], wv[2], wv[3]);
      }
   }
}

int launch_learn_features(Context* ctx, const float* e8, const float* u8, float* xf, const float* fstat,
   __nv_bfloat16* xn)
{
   PairParams P = make_params(ctx, DESC_CUT);
   k_learn_features<GROUP><<<grid_for((long long)ctx->npad * GROUP, PAIR_THREADS), PAIR_THREADS, 0, ctx->stream>>>(P,
      ctx->npad, ctx->cfg.cutoff >= DESC_CUT ? ctx->nbrc : ctx->nbr, ctx->cfg.cutoff >= DESC_CUT ? ctx->nnbrc : ctx->nnbr,
      ctx->sp_start, ctx->sp_j, ctx->sp_sc, ctx->spos, ctx->srpole, ctx->sframe, e8, u8, xf, ctx->spolar, fstat,
      ctx->status, xn);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}
}  // namespace t9gb
