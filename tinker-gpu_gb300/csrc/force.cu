// Multipole and polarization forces: real-space pair terms, the frame
// (torque) chain rule, and the final gradient.
//
// Formulation.  For every atom i the kernels accumulate
//  - the force at fixed global multipoles and fixed induced dipoles, and
//  - the "torque field" T_i = dE/dM_i: the derivative of the energy with
//    respect to atom i's global multipole (q, d, Theta), i.e. the potential,
//    its gradient and its second derivatives at i;
// the frame kernel then turns T_i into forces on the atoms that define i's
// local frame by differentiating the rotation M_i = A(x)^T M_local A(x)
// (forward-mode, one coordinate at a time).  This is the same physics as the
// reference's torque route (src/cu/amoeba/torque.cu:8-383 with the ufld /
// dufld and trq terms of include/seq/pair_mpole.h, pair_polar.h:39-366) in
// a different form, and reproduces its gradients
// (test/localframe.cpp:49-72, :133-151, :344-366, :521-543).
//
// Real space, pair i-k with R = x_i - x_k.  The potential tensor P of a
// source multipole (q, d, Theta) at the field point, with radial functions
// B_n (Ewald b_n of damp_ewald, include/seq/damp.h:136-151, or
// (2n-1)!!/r^(2n+1); m-scaled exclusions B_n - (1 - m) rr_n), is
//   p0  = q B0 + (d.R) B1 + (R.Theta.R) B2
//   p_a = d_a B1 + 2 (Theta R)_a B2 - R_a (q B1 + (d.R) B2 + (R.Theta.R) B3)
//   p_ab = R_a R_b c2 - delta_ab c1 - R_b w_a - R_a w_b + 2 Theta_ab B2
//   (c1 = q B1 + (d.R) B2 + (R.Theta.R) B3, c2 = q B2 + (d.R) B3 +
//    (R.Theta.R) B4, w_a = d_a B2 + 2 (Theta R)_a B3),
// with the quadrupole traces dropped as the reference's pair terms do, and
// the pair energy is M_i . P = q_i p0 + d_i . p1 + Theta_i : p2.  The
// derivatives with respect to R come from dual numbers whose radial parts
// use dB_n/dr = -r B_(n+1) exactly.
//
// Polarization (AMOEBA): the gradient at fixed dipoles of
//   G = -1/2 f [u_p . E_d + u_d . E_p + u_d . E_u(u_p)]
// (d-, p- and u-scaled Thole-damped fields; the damped B_n carry
// lambda_3/5/7 of damp_thole3 and their r-derivatives).  Per pair from i:
//   G_ik = 1/2 [u_p,i . p1^d(M_k) + u_d,i . p1^p(M_k)
//               + M_i . (P^d(u_p,k) + P^p(u_d,k))
//               + u_d,i . p1^u(u_p,k) + u_p,i . p1^u(u_d,k)]
// and dG/dM_i = 1/2 (P^d(u_p,k) + P^p(u_d,k)).
#include <cmath>

#include "pair.cuh"

namespace t9gb {

// ---------------------------------------------------------------------------
// dual numbers: value and gradient with respect to R

struct D3 {
   float v, x, y, z;
};

__device__ __forceinline__ D3 dc(float v) { return {v, 0.f, 0.f, 0.f}; }
__device__ __forceinline__ D3 operator+(D3 a, D3 b) { return {a.v + b.v, a.x + b.x, a.y + b.y, a.z + b.z}; }
__device__ __forceinline__ D3 operator-(D3 a, D3 b) { return {a.v - b.v, a.x - b.x, a.y - b.y, a.z - b.z}; }
__device__ __forceinline__ D3 operator*(D3 a, D3 b)
{
   return {a.v * b.v, a.x * b.v + a.v * b.x, a.y * b.v + a.v * b.y, a.z * b.v + a.v * b.z};
}
__device__ __forceinline__ D3 operator*(float s, D3 a) { return {s * a.v, s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ D3 operator*(D3 a, float s) { return {s * a.v, s * a.x, s * a.y, s * a.z}; }
__device__ __forceinline__ float val(float a) { return a; }
__device__ __forceinline__ float val(D3 a) { return a.v; }

// quadrupole storage: xx yy zz xy xz yz
struct Mp {
   float q, d[3], Q[6];
};

template <class T>
struct Pot {
   T p0, p1[3], p2[6];
};

__device__ __forceinline__ int q6(int a, int b)
{
   return a == b ? a : (a + b == 1 ? 3 : (a + b == 2 ? 4 : 5));
}

// potential tensor (p0, p1, p2) of source m; B[0..4]
template <class T>
__device__ __forceinline__ void source_pot(const T* R, const T* B, const Mp& m, Pot<T>& P)
{
   const T dR = R[0] * m.d[0] + R[1] * m.d[1] + R[2] * m.d[2];
   T QR[3];
#pragma unroll
   for (int a = 0; a < 3; ++a)
      QR[a] = R[0] * m.Q[q6(a, 0)] + R[1] * m.Q[q6(a, 1)] + R[2] * m.Q[q6(a, 2)];
   const T RQR = R[0] * QR[0] + R[1] * QR[1] + R[2] * QR[2];
   P.p0 = m.q * B[0] + dR * B[1] + RQR * B[2];
   const T c1 = m.q * B[1] + dR * B[2] + RQR * B[3];
   const T c2 = m.q * B[2] + dR * B[3] + RQR * B[4];
   T w[3];
#pragma unroll
   for (int a = 0; a < 3; ++a) {
      P.p1[a] = m.d[a] * B[1] + 2.f * QR[a] * B[2] - R[a] * c1;
      w[a] = m.d[a] * B[2] + 2.f * QR[a] * B[3];
   }
#pragma unroll
   for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = a; b < 3; ++b) {
         T v = R[a] * R[b] * c2 - R[b] * w[a] - R[a] * w[b] + 2.f * m.Q[q6(a, b)] * B[2];
         if (a == b)
            v = v - c1;
         P.p2[q6(a, b)] = v;
      }
}

// field-point gradient only (p1) of source m; B[1..3]
template <class T>
__device__ __forceinline__ void source_p1(const T* R, const T* B, const Mp& m, T* p1)
{
   const T dR = R[0] * m.d[0] + R[1] * m.d[1] + R[2] * m.d[2];
   T QR[3];
#pragma unroll
   for (int a = 0; a < 3; ++a)
      QR[a] = R[0] * m.Q[q6(a, 0)] + R[1] * m.Q[q6(a, 1)] + R[2] * m.Q[q6(a, 2)];
   const T RQR = R[0] * QR[0] + R[1] * QR[1] + R[2] * QR[2];
   const T c1 = m.q * B[1] + dR * B[2] + RQR * B[3];
#pragma unroll
   for (int a = 0; a < 3; ++a)
      p1[a] = m.d[a] * B[1] + 2.f * QR[a] * B[2] - R[a] * c1;
}

// dipole source: p0, p1, p2 with B[1..3]
template <class T>
__device__ __forceinline__ void dipole_pot(const T* R, const T* B, const float* u, Pot<T>& P)
{
   const T dR = R[0] * u[0] + R[1] * u[1] + R[2] * u[2];
   P.p0 = dR * B[1];
   const T c1 = dR * B[2];
   const T c2 = dR * B[3];
   T w[3];
#pragma unroll
   for (int a = 0; a < 3; ++a) {
      P.p1[a] = u[a] * B[1] - R[a] * c1;
      w[a] = u[a] * B[2];
   }
#pragma unroll
   for (int a = 0; a < 3; ++a)
#pragma unroll
      for (int b = a; b < 3; ++b) {
         T v = R[a] * R[b] * c2 - R[b] * w[a] - R[a] * w[b];
         if (a == b)
            v = v - c1;
         P.p2[q6(a, b)] = v;
      }
}

template <class T>
__device__ __forceinline__ void dipole_p1(const T* R, const T* B, const float* u, T* p1)
{
   const T dR = R[0] * u[0] + R[1] * u[1] + R[2] * u[2];
   const T c1 = dR * B[2];
#pragma unroll
   for (int a = 0; a < 3; ++a)
      p1[a] = u[a] * B[1] - R[a] * c1;
}

// M . P
template <class T>
__device__ __forceinline__ T contract(const Mp& m, const Pot<T>& P)
{
   T e = m.q * P.p0 + m.d[0] * P.p1[0] + m.d[1] * P.p1[1] + m.d[2] * P.p1[2];
   e = e + m.Q[0] * P.p2[0] + m.Q[1] * P.p2[1] + m.Q[2] * P.p2[2];
   e = e + 2.f * (m.Q[3] * P.p2[3] + m.Q[4] * P.p2[4] + m.Q[5] * P.p2[5]);
   return e;
}

__device__ __forceinline__ void load_mp(const float* __restrict__ rp, int s, Mp& m)
{
   const float* r = rp + 12 * s;
   m.q = r[0];
   m.d[0] = r[1];
   m.d[1] = r[2];
   m.d[2] = r[3];
#pragma unroll
   for (int c = 0; c < 6; ++c)
      m.Q[c] = r[4 + c];
}

// Ewald (or bare) b_0..b_5 and bare rr_0..rr_5 at r
__device__ __forceinline__ void radial(const PairParams& P, float r, float* bn, float* rr)
{
   const float invr = 1.f / r, rr2 = invr * invr;
   rr[0] = invr;
#pragma unroll
   for (int n = 1; n <= 5; ++n)
      rr[n] = (2 * n - 1) * rr[n - 1] * rr2;
   if (P.ewald) {
      const float ra = P.aewald * r;
      const float ex = __expf(-ra * ra);
      bn[0] = erfc_hastings(ra, ex) * invr;
      float alsq2n = 1.f / (1.77245385f * P.aewald);
      const float alsq2 = 2.f * P.aewald * P.aewald;
#pragma unroll
      for (int n = 1; n <= 5; ++n) {
         alsq2n *= alsq2;
         bn[n] = ((2 * n - 1) * bn[n - 1] + alsq2n * ex) * rr2;
      }
   } else {
#pragma unroll
      for (int n = 0; n <= 5; ++n)
         bn[n] = rr[n];
   }
}

// per-lane partial sums over the lane's few pairs (FP32); the lanes of an
// atom are combined in FP64
struct PairOut {
   float e;      // empole pair energy (i side, halved later)
   float f[3];   // force on i
   float t[10];  // torque field at i
   float w[9];   // virial dE/d(strain)_ab, i side of the pair (halved)
};

// one pair seen from i: R = x_i - x_k, scales sc = (m, d, p, u)
template <bool MPOLE, bool POLAR, bool VIR>
__device__ __forceinline__ void elec_pair(const PairParams& P, float3 Rv, float r2, float4 sc, const Mp& mi,
   const float* ui, float pdi, float pti, const Mp& mk, const float* uk, float pdk, float ptk, PairOut& o)
{
   const float r = sqrtf(r2);
   float bn[6], rr[6];
   radial(P, r, bn, rr);
   const D3 R[3] = {{Rv.x, 1.f, 0.f, 0.f}, {Rv.y, 0.f, 1.f, 0.f}, {Rv.z, 0.f, 0.f, 1.f}};
   if (MPOLE) {
      // m-scaled radial functions and their duals (dB_n = -B_(n+1) R)
      float B[6];
#pragma unroll
      for (int n = 0; n <= 5; ++n)
         B[n] = bn[n] - (1.f - sc.x) * rr[n];
      D3 Bd[5];
#pragma unroll
      for (int n = 0; n < 5; ++n)
         Bd[n] = {B[n], -B[n + 1] * Rv.x, -B[n + 1] * Rv.y, -B[n + 1] * Rv.z};
      Pot<D3> pk;
      source_pot(R, Bd, mk, pk);
      const D3 e = contract(mi, pk);
      o.e += e.v;
      o.f[0] -= e.x;
      o.f[1] -= e.y;
      o.f[2] -= e.z;
      if (VIR) {
         const float ge[3] = {e.x, e.y, e.z}, rv[3] = {Rv.x, Rv.y, Rv.z};
#pragma unroll
         for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
               o.w[3 * a + b] += 0.5f * ge[a] * rv[b];
      }
      o.t[0] += pk.p0.v;
#pragma unroll
      for (int a = 0; a < 3; ++a)
         o.t[1 + a] += pk.p1[a].v;
#pragma unroll
      for (int c = 0; c < 6; ++c)
         o.t[4 + c] += pk.p2[c].v;
   }
   if (POLAR) {
      // Thole damping lambda_3/5/7 and d lambda / dr
      const float pg = pair_gamma(P, pti, ptk);
      const float dmp = pdi * pdk;
      float a = 0.f, ea = 0.f;
      if (dmp != 0.f) {
         const float ratio = r / dmp;
         a = pg * ratio * ratio * ratio;
         ea = __expf(-a);
      }
      const float lam[3] = {1.f - ea, 1.f - (1.f + a) * ea, 1.f - (1.f + a + 0.6f * a * a) * ea};
      const float ir = 1.f / r;
      const float dlam[3] = {ea == 0.f ? 0.f : 3.f * a * ea * ir, ea == 0.f ? 0.f : 3.f * a * a * ea * ir,
         ea == 0.f ? 0.f : (1.8f * a * a * a - 0.6f * a * a) * ea * ir};
      // damped duals for the d, p, u scales: index n = 1..3 in B[n]
      D3 Bs[3][5];
      const float sv[3] = {sc.y, sc.z, sc.w};
#pragma unroll
      for (int k = 0; k < 3; ++k) {
         Bs[k][0] = dc(0.f);
         Bs[k][4] = dc(0.f);
#pragma unroll
         for (int n = 1; n <= 3; ++n) {
            const float sl = sv[k] * lam[n - 1];
            const float D = bn[n] - (1.f - sl) * rr[n];
            const float g = -bn[n + 1] + sv[k] * dlam[n - 1] * rr[n] * ir + (1.f - sl) * rr[n + 1];
            Bs[k][n] = {D, g * Rv.x, g * Rv.y, g * Rv.z};
         }
      }
      const float* udi = ui;
      const float* upi = ui + 3;
      const float* udk = uk;
      const float* upk = uk + 3;
      D3 p1[3];
      // u_p,i . p1^d(M_k) + u_d,i . p1^p(M_k)
      source_p1(R, Bs[0], mk, p1);
      D3 g = upi[0] * p1[0] + upi[1] * p1[1] + upi[2] * p1[2];
      source_p1(R, Bs[1], mk, p1);
      g = g + udi[0] * p1[0] + udi[1] * p1[1] + udi[2] * p1[2];
      // M_i . (P^d(u_p,k) + P^p(u_d,k))
      Pot<D3> pa, pb;
      dipole_pot(R, Bs[0], upk, pa);
      dipole_pot(R, Bs[1], udk, pb);
      g = g + contract(mi, pa) + contract(mi, pb);
      // mutual
      dipole_p1(R, Bs[2], upk, p1);
      g = g + udi[0] * p1[0] + udi[1] * p1[1] + udi[2] * p1[2];
      dipole_p1(R, Bs[2], udk, p1);
      g = g + upi[0] * p1[0] + upi[1] * p1[1] + upi[2] * p1[2];
      o.f[0] -= 0.5f * g.x;
      o.f[1] -= 0.5f * g.y;
      o.f[2] -= 0.5f * g.z;
      if (VIR) {
         const float gg[3] = {g.x, g.y, g.z}, rv[3] = {Rv.x, Rv.y, Rv.z};
#pragma unroll
         for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
               o.w[3 * a + b] += 0.25f * gg[a] * rv[b];
      }
      o.t[0] += 0.5f * (pa.p0.v + pb.p0.v);
#pragma unroll
      for (int c = 0; c < 3; ++c)
         o.t[1 + c] += 0.5f * (pa.p1[c].v + pb.p1[c].v);
#pragma unroll
      for (int c = 0; c < 6; ++c)
         o.t[4 + c] += 0.5f * (pa.p2[c].v + pb.p2[c].v);
   }
}

// Real-space forces and torque fields, G lanes per atom i over the list and
// the scaled partners.  f: electric; outputs per slot: force [npad][3],
// torque field [npad][10], empole real energy (MPOLE).
template <int G, bool MPOLE, bool POLAR, bool VIR>
__global__ void __launch_bounds__(128) k_elec_real(PairParams P, int npad, float f, const int* __restrict__ nbr,
   const int* __restrict__ nnbr, const int* __restrict__ sp_start, const int* __restrict__ sp_j,
   const float4* __restrict__ sp_sc, const float4* __restrict__ spos, const float* __restrict__ rp,
   const float* __restrict__ u8, float* __restrict__ fout, float* __restrict__ tout, double* __restrict__ e_atom,
   float* __restrict__ wout)
{
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid / G, g = tid % G;
   if (i >= npad)
      return;
   PairOut o;
   o.e = 0;
   o.f[0] = o.f[1] = o.f[2] = 0;
#pragma unroll
   for (int c = 0; c < 10; ++c)
      o.t[c] = 0;
#pragma unroll
   for (int c = 0; c < 9; ++c)
      o.w[c] = 0;
   if (i < P.n) {
      const float4 pi = spos[i];
      Mp mi;
      load_mp(rp, i, mi);
      float ui[8] = {0, 0, 0, 0, 0, 0, 0, 0};
      if (POLAR)
         load8(u8, i, ui);
      const float pti = rp[12 * i + 10];
      const int* row = nbr + (size_t)i * P.cap;
      const int cnt = nnbr[i];
      for (int k = g; k < cnt; k += G) {
         const int j = row[k];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            Mp mk;
            load_mp(rp, j, mk);
            float uk[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (POLAR)
               load8(u8, j, uk);
            elec_pair<MPOLE, POLAR, VIR>(P, make_float3(-d.x, -d.y, -d.z), r2, make_float4(1.f, 1.f, 1.f, 1.f), mi, ui,
               pi.w, pti, mk, uk, pk.w, rp[12 * j + 10], o);
         }
      }
      const int pa = sp_start[i], pb = sp_start[i + 1];
      for (int q = pa + g; q < pb; q += G) {
         const int j = sp_j[q];
         const float4 pk = spos[j];
         const float3 d = sep(P, pi, pk);
         const float r2 = d.x * d.x + d.y * d.y + d.z * d.z;
         if (r2 <= P.cut2) {
            Mp mk;
            load_mp(rp, j, mk);
            float uk[8] = {0, 0, 0, 0, 0, 0, 0, 0};
            if (POLAR)
               load8(u8, j, uk);
            elec_pair<MPOLE, POLAR, VIR>(P, make_float3(-d.x, -d.y, -d.z), r2, sp_sc[q], mi, ui, pi.w, pti, mk, uk, pk.w,
               rp[12 * j + 10], o);
         }
      }
   }
   // the lane partials are FP32: their group sum stays FP32 (this GPU's FP64
   // pipe is far narrower), the outputs are scaled from it
   float acc[14];
   acc[0] = o.e;
   acc[1] = o.f[0];
   acc[2] = o.f[1];
   acc[3] = o.f[2];
#pragma unroll
   for (int c = 0; c < 10; ++c)
      acc[4 + c] = o.t[c];
   group_reduce<G, 14>(acc);
   float wv[9];
   if (VIR) {
#pragma unroll
      for (int c = 0; c < 9; ++c)
         wv[c] = o.w[c];
      group_reduce<G, 9>(wv);
   }
   if (g == 0) {
      if (VIR)
#pragma unroll
         for (int c = 0; c < 9; ++c)
            wout[c * npad + i] = f * wv[c];
      if (MPOLE && e_atom)
         e_atom[i] = 0.5 * (double)f * (double)acc[0];
#pragma unroll
      for (int c = 0; c < 3; ++c)
         fout[3 * i + c] = f * acc[1 + c];
#pragma unroll
      for (int c = 0; c < 10; ++c)
         tout[10 * i + c] = f * acc[4 + c];
   }
}

// ---------------------------------------------------------------------------
// frame chain rule: forces on the frame atoms from the torque field

struct D1 {
   float v, d;
};
__device__ __forceinline__ D1 operator+(D1 a, D1 b) { return {a.v + b.v, a.d + b.d}; }
__device__ __forceinline__ D1 operator-(D1 a, D1 b) { return {a.v - b.v, a.d - b.d}; }
__device__ __forceinline__ D1 operator*(D1 a, D1 b) { return {a.v * b.v, a.d * b.v + a.v * b.d}; }

__device__ __forceinline__ void norm3(D1* v)
{
   const D1 s = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
   const float inv = rsqrtf(s.v);
   const D1 w = {inv, -0.5f * s.d * inv * inv * inv};
   v[0] = v[0] * w;
   v[1] = v[1] * w;
   v[2] = v[2] * w;
}

// The rotation of k_rotpole (rows x, y, z axes) and its derivative along one
// coordinate: role r (0 atom i, 1 z atom, 2 x atom, 3 y atom), component c.
__device__ void frame_rot(const float* xi, const float* xz, const float* xx, const float* xy, int kind, int role,
   int comp, D1 A[3][3])
{
   auto diff = [&](const float* p, int prole, D1* v) {
#pragma unroll
      for (int c = 0; c < 3; ++c) {
         float dv = 0.f;
         if (c == comp) {
            if (role == prole)
               dv += 1.f;
            if (role == 0)
               dv -= 1.f;
         }
         v[c] = {p[c] - xi[c], dv};
      }
   };
   D1* X = A[0];
   D1* Y = A[1];
   D1* Z = A[2];
   diff(xz, 1, Z);
   norm3(Z);
   if (kind == 1) {
      const bool okay = !(fabsf(Z[0].v) > 0.866f);
      X[0] = {okay ? 1.f : 0.f, 0.f};
      X[1] = {okay ? 0.f : 1.f, 0.f};
      X[2] = {0.f, 0.f};
   } else {
      diff(xx, 2, X);
      norm3(X);
   }
   if (kind == 4 || kind == 5) {
      diff(xy, 3, Y);
      norm3(Y);
   }
   if (kind == 3) {
      for (int d = 0; d < 3; ++d)
         Z[d] = Z[d] + X[d];
      norm3(Z);
   } else if (kind == 4) {
      for (int d = 0; d < 3; ++d)
         X[d] = X[d] + Y[d];
      norm3(X);
   } else if (kind == 5) {
      for (int d = 0; d < 3; ++d)
         Z[d] = Z[d] + X[d] + Y[d];
      norm3(Z);
   }
   const D1 dot = X[0] * Z[0] + X[1] * Z[1] + X[2] * Z[2];
   for (int d = 0; d < 3; ++d)
      X[d] = X[d] - dot * Z[d];
   norm3(X);
   Y[0] = X[2] * Z[1] - X[1] * Z[2];
   Y[1] = X[0] * Z[2] - X[2] * Z[0];
   Y[2] = X[1] * Z[0] - X[0] * Z[1];
}

// fbuf[s][3 role + c] = -dE/dx(role atom, c) through the rotation of slot s
// wout (may be null): the frame part of the virial, -sum_role F_role (x_role - x_i)
__global__ void k_frame_force(int npad, const int* __restrict__ perm, const int4* __restrict__ frames,
   const float* __restrict__ pole, const float* __restrict__ xyz, const float* __restrict__ t0,
   const float* __restrict__ t1, const float* __restrict__ t2, float* __restrict__ fbuf, float* __restrict__ wout)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      float* out = fbuf + 12 * s;
      for (int m = 0; m < 12; ++m)
         out[m] = 0.f;
      if (wout)
         for (int c = 0; c < 9; ++c)
            wout[c * npad + s] = 0.f;
      const int i = perm[s];
      if (i < 0)
         continue;
      const int4 f = frames[i];
      if (f.w == 0)
         continue;
      float T[10];
      for (int c = 0; c < 10; ++c)
         T[c] = t0[10 * s + c] + (t1 ? t1[10 * s + c] : 0.f) + (t2 ? t2[10 * s + c] : 0.f);
      const float* p = pole + 10 * i;
      const float Ql[3][3] = {{p[4], p[7], p[8]}, {p[7], p[5], p[9]}, {p[8], p[9], p[6]}};
      float T2[3][3];
      for (int a = 0; a < 3; ++a)
         for (int b = 0; b < 3; ++b)
            T2[a][b] = T[4 + q6(a, b)];
      const float* xi = xyz + 3 * i;
      const float* xz = xyz + 3 * f.x;
      const float* xx = f.w == 1 ? xi : xyz + 3 * f.y;
      const int iy = abs(f.z) - 1;
      const float* xy = (f.w == 4 || f.w == 5) ? xyz + 3 * iy : xi;
      const int nrole = (f.w == 4 || f.w == 5) ? 4 : (f.w == 1 ? 2 : 3);
      for (int role = 0; role < nrole; ++role)
         for (int c = 0; c < 3; ++c) {
            D1 A[3][3];
            frame_rot(xi, xz, xx, xy, f.w, role, c, A);
            float dE = 0.f;
            // d_glob,c = sum_j p[1+j] A[j][c]
            for (int cc = 0; cc < 3; ++cc) {
               float dd = 0.f;
               for (int j = 0; j < 3; ++j)
                  dd += p[1 + j] * A[j][cc].d;
               dE += T[1 + cc] * dd;
            }
            // Theta_glob,cd = sum_jk A[j][c] Ql[j][k] A[k][d]
            for (int cc = 0; cc < 3; ++cc)
               for (int dd = 0; dd < 3; ++dd) {
                  float dq = 0.f;
                  for (int j = 0; j < 3; ++j)
                     for (int k = 0; k < 3; ++k)
                        dq += Ql[j][k] * (A[j][cc].d * A[k][dd].v + A[j][cc].v * A[k][dd].d);
                  dE += T2[cc][dd] * dq;
               }
            out[3 * role + c] = -dE;
         }
      if (wout) {
         const float* pos[4] = {xi, xz, xx, xy};
         for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b) {
               float w = 0.f;
               for (int role = 1; role < nrole; ++role)
                  w -= out[3 * role + a] * (pos[role][b] - xi[b]);
               wout[(3 * a + b) * npad + s] = w;
            }
      }
   }
}

// Permanent multipoles in a uniform external field E (e/A^2): energy
// -f (q r.E + d.E) per atom at the caller's coordinates, force f q E, torque
// field dE/dd = -f E (the frame chain rule turns it into frame forces), and
// virial rows dE/d(eps_ab) = -f q E_a r_b (exfieldDipole_cu1,
// src/cu/amoeba/empole.cu:79-130).  Adds to what the pair and reciprocal
// kernels stored; any output may be null.
__global__ void k_extfield_mpole(int npad, const int* __restrict__ perm, const float* __restrict__ xyz,
   const float* __restrict__ rp, float e0, float e1, float e2, float f, float* __restrict__ fout,
   float* __restrict__ tout, float* __restrict__ wout, double* __restrict__ e_one)
{
   for (int s = blockIdx.x * blockDim.x + threadIdx.x; s < npad; s += gridDim.x * blockDim.x) {
      const int i = perm[s];
      if (i < 0)
         continue;
      const float E[3] = {e0, e1, e2};
      const float r[3] = {xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
      const float* m = rp + 12 * s;
      const float rE = r[0] * E[0] + r[1] * E[1] + r[2] * E[2];
      if (e_one)
         e_one[s] += -(double)f * ((double)m[0] * rE + (double)m[1] * E[0] + (double)m[2] * E[1] + (double)m[3] * E[2]);
      if (fout)
         for (int c = 0; c < 3; ++c)
            fout[3 * s + c] += f * m[0] * E[c];
      if (tout) {
         tout[10 * s] += -f * rE;
         for (int c = 0; c < 3; ++c)
            tout[10 * s + 1 + c] += -f * E[c];
      }
      if (wout)
         for (int a = 0; a < 3; ++a)
            for (int b = 0; b < 3; ++b)
               wout[(3 * a + b) * npad + s] += -f * m[0] * E[a] * r[b];
   }
}

int launch_extfield_mpole(Context* ctx, bool forces, bool vir)
{
   if (!ctx->use_exfld)
      return T9GB_OK;
   const float* E = ctx->h_exfld;
   k_extfield_mpole<<<grid_for(ctx->npad, 256), 256, 0, ctx->stream>>>(ctx->npad, ctx->perm, ctx->xyz, ctx->srpole,
      E[0], E[1], E[2], (float)ctx->cfg.electric, forces ? ctx->freal : nullptr, forces ? ctx->treal : nullptr,
      vir ? ctx->wvir : nullptr, ctx->e_atom + 2 * (size_t)ctx->npad);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// gradient (caller order) = -(sum of the per-slot forces + frame forces)
__global__ void k_force_combine(int n, const int* __restrict__ iperm, const float* __restrict__ f0,
   const float* __restrict__ f1, const float* __restrict__ f2, const int* __restrict__ rev_start,
   const int* __restrict__ rev_ent, const float* __restrict__ fbuf, float* __restrict__ grad)
{
   for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
      const int s = iperm[a];
      float F[3];  // FP32, like the gradient it becomes
      for (int c = 0; c < 3; ++c)
         F[c] = f0[3 * s + c] + (f1 ? f1[3 * s + c] : 0.f) + (f2 ? f2[3 * s + c] : 0.f);
      for (int e = rev_start[s]; e < rev_start[s + 1]; ++e) {
         const int ent = rev_ent[e];
         const float* fb = fbuf + 12 * (ent >> 2) + 3 * (ent & 3);
         for (int c = 0; c < 3; ++c)
            F[c] += fb[c];
      }
      for (int c = 0; c < 3; ++c)
         grad[3 * a + c] = -F[c];
   }
}

// ---------------------------------------------------------------------------

int force_setup(Context* ctx)
{
   if (ctx->freal)
      return T9GB_OK;
   const size_t np = ctx->npad;
   T9_CUDA(cudaMalloc(&ctx->freal, sizeof(float) * 3 * np));
   T9_CUDA(cudaMalloc(&ctx->frecp, sizeof(float) * 3 * np));
   T9_CUDA(cudaMalloc(&ctx->frecu, sizeof(float) * 3 * np));
   T9_CUDA(cudaMalloc(&ctx->treal, sizeof(float) * 10 * np));
   T9_CUDA(cudaMalloc(&ctx->trecp, sizeof(float) * 10 * np));
   T9_CUDA(cudaMalloc(&ctx->trecu, sizeof(float) * 10 * np));
   T9_CUDA(cudaMalloc(&ctx->fbuf, sizeof(float) * 12 * np));
   T9_CUDA(cudaMalloc(&ctx->wvir, sizeof(float) * 27 * np));
   T9_CUDA(cudaMalloc(&ctx->vsum, sizeof(double) * 32));
   return T9GB_OK;
}

void force_free(Context* ctx)
{
   void* p[] = {ctx->freal, ctx->frecp, ctx->frecu, ctx->treal, ctx->trecp, ctx->trecu, ctx->fbuf, ctx->rev_start,
      ctx->rev_ent, ctx->wvir, ctx->vsum};
   for (void* q : p)
      if (q)
         cudaFree(q);
   ctx->freal = ctx->frecp = ctx->frecu = ctx->treal = ctx->trecp = ctx->trecu = ctx->fbuf = nullptr;
   ctx->rev_start = ctx->rev_ent = nullptr;
   ctx->wvir = nullptr;
   ctx->vsum = nullptr;
}

// reverse frame map: for slot j, the (slot i, role) pairs whose frame uses j
int frame_map_build(Context* ctx)
{
   const int n = ctx->n, npad = ctx->npad;
   std::vector<std::vector<int>> ent(npad);
   for (int a = 0; a < n; ++a) {
      const int s = ctx->h_iperm[a];
      const int* f = &ctx->h_frames[4 * a];
      ent[s].push_back(4 * s + 0);
      if (f[3] == 0)
         continue;
      ent[ctx->h_iperm[f[0]]].push_back(4 * s + 1);
      if (f[3] != 1)
         ent[ctx->h_iperm[f[1]]].push_back(4 * s + 2);
      if (f[3] == 4 || f[3] == 5)
         ent[ctx->h_iperm[std::abs(f[2]) - 1]].push_back(4 * s + 3);
   }
   std::vector<int> start(npad + 1, 0), flat;
   for (int j = 0; j < npad; ++j) {
      start[j + 1] = start[j] + (int)ent[j].size();
      flat.insert(flat.end(), ent[j].begin(), ent[j].end());
   }
   if (ctx->rev_start)
      cudaFree(ctx->rev_start);
   if (ctx->rev_ent)
      cudaFree(ctx->rev_ent);
   T9_CUDA(cudaMalloc(&ctx->rev_start, sizeof(int) * (npad + 1)));
   T9_CUDA(cudaMalloc(&ctx->rev_ent, sizeof(int) * std::max<size_t>(1, flat.size())));
   T9_CUDA(cudaMemcpyAsync(ctx->rev_start, start.data(), sizeof(int) * (npad + 1), cudaMemcpyHostToDevice,
      ctx->stream));
   if (!flat.empty())
      T9_CUDA(cudaMemcpyAsync(ctx->rev_ent, flat.data(), sizeof(int) * flat.size(), cudaMemcpyHostToDevice,
         ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return T9GB_OK;
}

// Forces of the permanent multipoles (mpole) and/or of the polarization at
// the last induce's dipoles (polar).  grad: caller order [n][3] device.
// e_atom receives the multipole energy terms (real, recip, self) when mpole.
// vir: per-slot virial rows wvir [27][npad] (real, frame, reciprocal) and the
// k-space sums in scal[40..51].
template <int G, bool MPOLE, bool POLAR, bool VIR>
static void launch_real_g(Context* ctx, const PairParams& P, float f)
{
   const int grid = grid_for((long long)ctx->npad * G, 128);
   k_elec_real<G, MPOLE, POLAR, VIR><<<grid, 128, 0, ctx->stream>>>(P, ctx->npad, f, ctx->nbrc, ctx->nnbrc,
      ctx->sp_start, ctx->sp_j, ctx->sp_sc, ctx->spos, ctx->srpole, ctx->uind, ctx->freal, ctx->treal,
      MPOLE ? ctx->e_atom : nullptr, ctx->wvir);
}

// lanes per atom: t9gb_force_lanes (4, 8 or 16)
template <bool MPOLE, bool POLAR, bool VIR>
static void launch_real(Context* ctx, const PairParams& P, float f)
{
   if (ctx->force_lanes == 4)
      launch_real_g<4, MPOLE, POLAR, VIR>(ctx, P, f);
   else if (ctx->force_lanes == 8)
      launch_real_g<8, MPOLE, POLAR, VIR>(ctx, P, f);
   else
      launch_real_g<16, MPOLE, POLAR, VIR>(ctx, P, f);
}

// the second reciprocal half needs the third side stream (eager calls only:
// inside a graph capture the side streams belong to the capture levels)
static bool two_halves_ok(const Context* ctx)
{
   return ctx->side_stream[2] != nullptr && ctx->pme.qgrid2 != nullptr && side_index(ctx) == 0;
}

int elec_forces(Context* ctx, bool mpole, bool polar, float* grad, bool vir)
{
   T9_CHECK(force_setup(ctx));
   if (!ctx->rev_start)
      T9_CHECK(frame_map_build(ctx));
   const PairParams P = make_params(ctx, ctx->cfg.cutoff);
   const float f = (float)ctx->cfg.electric;
   const bool ew = ctx->cfg.use_ewald != 0;
   const size_t np = ctx->npad;
   float* wrec = vir ? ctx->wvir + 18 * np : nullptr;
   // the reciprocal forces (spread, transform, gather: their own outputs)
   // run on side streams beside the real-space kernel; without the virial
   // the permanent and the induced-dipole halves run beside each other too
   // (the dipole half on the second grid)
   const bool side = ew && !ctx->prof.on;
   const bool two = side && polar && !vir && two_halves_ok(ctx);
   const int k = side_index(ctx);
   if (side) {
      T9_CHECK(recip_fork(ctx, k));
      if (two)
         T9_CHECK(recip_fork(ctx, 2));
      cudaStream_t main = ctx->stream;
      ctx->stream = ctx->side_stream[k];
      int rc = two ? launch_force_recip_perm(ctx, mpole, polar, wrec) : launch_force_recip(ctx, mpole, polar, wrec);
      if (rc == T9GB_OK && two) {
         ctx->stream = ctx->side_stream[2];
         rc = launch_force_recip_uind(ctx, wrec, true);
      }
      ctx->stream = main;
      T9_CHECK(rc);
   }
   if (vir) {
      if (mpole && polar)
         launch_real<true, true, true>(ctx, P, f);
      else if (mpole)
         launch_real<true, false, true>(ctx, P, f);
      else
         launch_real<false, true, true>(ctx, P, f);
   } else {
      if (mpole && polar)
         launch_real<true, true, false>(ctx, P, f);
      else if (mpole)
         launch_real<true, false, false>(ctx, P, f);
      else
         launch_real<false, true, false>(ctx, P, f);
   }
   T9_CUDA(cudaGetLastError());
   if (side) {
      T9_CHECK(recip_join(ctx, k));
      if (two)
         T9_CHECK(recip_join(ctx, 2));
   }
   else if (ew)
      T9_CHECK(launch_force_recip(ctx, mpole, polar, wrec));
   else if (vir)
      T9_CUDA(cudaMemsetAsync(ctx->wvir + 18 * np, 0, sizeof(float) * 9 * np, ctx->stream));
   if (mpole)
      T9_CHECK(launch_extfield_mpole(ctx, true, vir));
   k_frame_force<<<grid_for(ctx->npad, 128), 128, 0, ctx->stream>>>(ctx->npad, ctx->perm, ctx->frames, ctx->pole,
      ctx->xyz, ctx->treal, ew ? ctx->trecp : nullptr, ew && polar ? ctx->trecu : nullptr, ctx->fbuf,
      vir ? ctx->wvir + 9 * np : nullptr);
   if (grad)
      k_force_combine<<<grid_for(ctx->n, 128), 128, 0, ctx->stream>>>(ctx->n, ctx->iperm, ctx->freal,
         ew ? ctx->frecp : nullptr, ew && polar ? ctx->frecu : nullptr, ctx->rev_start, ctx->rev_ent, ctx->fbuf, grad);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

}  // namespace t9gb
