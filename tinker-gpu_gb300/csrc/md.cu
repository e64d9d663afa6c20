// Molecular dynamics around induce(): velocity Verlet with an optional Bussi
// thermostat, forces from the multipole + polarization terms (t9gb_emplar's
// path, induce included), the buffered 14-7 van der Waals and the valence
// terms, whichever the context holds.
//
// Restates the reference's VerletIntegrator (src/md/integrator.cpp:70-190:
// KickOff energy, vel1(dt/2), pos(dt), energy, vel2(dt/2), thermostat
// control2) and bussiThermostat (src/mdpt.cpp:41-71).  Positions and
// velocities are FP64 on the device (caller order); forces come in FP32 as
// in the reference's mixed build.  a = -g / m * ekcal, ekcal = 418.4
// (kcal/mol -> g/mol A^2/ps^2).
#include "common.cuh"
#include "reduce.cuh"

#include <algorithm>
#include <cmath>
#include <random>

namespace t9gb {

constexpr double EKCAL = 418.4;
constexpr double GASCONST = 1.987204259e-3;  // kcal/mol/K (Tinker's units::gasconst)

// v += -g ekcal / m * h
// v -= h g / m for the gradient g + g2 (g2: the van der Waals and valence
// part, computed beside the electrostatic forces; may be null)
__global__ void k_md_kick(int n, double h, const float* __restrict__ g, const float* __restrict__ g2,
   const double* __restrict__ minv, double* __restrict__ v)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 3 * n; e += gridDim.x * blockDim.x) {
      const double gt = g2 ? (double)g[e] + (double)g2[e] : (double)g[e];
      v[e] -= h * EKCAL * minv[e / 3] * gt;
   }
}

// the step's total gradient g + g2 (g2 may be null)
__global__ void k_md_grad_total(int n, const float* __restrict__ g, const float* __restrict__ g2,
   float* __restrict__ out)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 3 * n; e += gridDim.x * blockDim.x)
      out[e] = g2 ? g[e] + g2[e] : g[e];
}

// x += v dt; the force kernels' float copy
__global__ void k_md_drift(int n, double dt, const double* __restrict__ v, double* __restrict__ x,
   float* __restrict__ xf)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 3 * n; e += gridDim.x * blockDim.x) {
      const double y = x[e] + dt * v[e];
      x[e] = y;
      xf[e] = (float)y;
   }
}

// 1/2 sum m v^2 (g/mol A^2/ps^2), fixed order: block partials then one block
__global__ void k_md_kinetic(int n, const double* __restrict__ v, const double* __restrict__ minv,
   double* __restrict__ red, double* __restrict__ out, int* __restrict__ ticket)
{
   __shared__ double sh[64];
   float s = 0.f;  // FP32 per thread and warp, FP64 above
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
      const double* w = v + 3 * i;
      const float x = (float)w[0], y = (float)w[1], z = (float)w[2];
      s += (x * x + y * y + z * z) / (float)minv[i];
   }
   const float pv[1] = {s};
   store_partials_f<1>(red, 0, pv, sh);
   if (!last_block(ticket))
      return;
   double t[1];
   sum_slots(red, 0, 1, gridDim.x, sh, t);
   if (threadIdx.x == 0)
      *out = 0.5 * t[0];
}

// Bussi factor of one step from the kinetic energy in md_out[0] and the
// step's variates (normal r, chi-squared s), stored in md_out[1]
__global__ void k_md_bussi(const double* __restrict__ rs, int step, double c, double kelvin, int nfree,
   double* __restrict__ out)
{
   const double ek = out[0] / EKCAL;
   double temp = 2.0 * ek / (nfree * GASCONST);
   if (temp == 0)
      temp = 0.1;
   const double d = (1 - c) * (kelvin / temp) / nfree;
   const double r = rs[2 * step], s = rs[2 * step + 1];
   double scale = sqrt(c + (s + r * r) * d + 2 * r * sqrt(c * d));
   if (r + sqrt(c / d) < 0)
      scale = -scale;
   out[1] = scale;
}

__global__ void k_md_scale(int n, const double* __restrict__ s, double* __restrict__ v)
{
   const double f = *s;
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < 3 * n; e += gridDim.x * blockDim.x)
      v[e] *= f;
}

static int md_free(Context* ctx)
{
   void* p[] = {ctx->md_x, ctx->md_v, ctx->md_minv, ctx->md_g, ctx->md_g2, ctx->md_red, ctx->md_out, ctx->md_rs};
   for (void* q : p)
      if (q)
         cudaFree(q);
   ctx->md_x = ctx->md_v = ctx->md_minv = ctx->md_red = ctx->md_out = nullptr;
   ctx->md_g = ctx->md_g2 = nullptr;
   ctx->md_rs = nullptr;
   ctx->md_rs_cap = 0;
   ctx->md_ready = false;
   return T9GB_OK;
}

void md_release(Context* ctx) { md_free(ctx); }

// gradient at ctx->xyz: electrostatics into md_g and, on side stream 3
// beside the electrostatic forces (after the dipole solve, with the list
// fixed), the van der Waals and valence terms into md_g2; the kicks add them
static int md_forces(Context* ctx, t9gb_context* h)
{
   (void)h;
   T9_CHECK(scatter_positions(ctx));
   T9_CHECK(rotpole_sorted(ctx));
   const bool extra = ctx->use_vdw || ctx->nval > 0;
   if (extra)
      T9_CUDA(cudaMemsetAsync(ctx->md_g2, 0, sizeof(float) * 3 * ctx->n, ctx->stream));
   bool forked = false;
   const std::function<int()> beside = [&]() -> int {
      if (!extra)
         return T9GB_OK;
      T9_CUDA(cudaEventRecord(ctx->ev_fork[3], ctx->stream));
      T9_CUDA(cudaStreamWaitEvent(ctx->side_stream[3], ctx->ev_fork[3], 0));
      forked = true;
      cudaStream_t main = ctx->stream;
      ctx->stream = ctx->side_stream[3];
      int rc = vdw_forces(ctx, ctx->md_g2, true, false, nullptr);
      if (rc == T9GB_OK)
         rc = valence_forces(ctx, ctx->md_g2, true, false);
      ctx->stream = main;
      return rc;
   };
   const std::function<int()> reset = [&]() -> int {
      if (forked) {  // the first pass's beside work ends before it is redone
         T9_CUDA(cudaEventRecord(ctx->ev_join[3], ctx->side_stream[3]));
         T9_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_join[3], 0));
      }
      if (extra)
         T9_CUDA(cudaMemsetAsync(ctx->md_g2, 0, sizeof(float) * 3 * ctx->n, ctx->stream));
      return T9GB_OK;
   };
   const int st = emplar_grad_beside(ctx, ctx->md_g, beside, reset);
   if (forked) {
      T9_CUDA(cudaEventRecord(ctx->ev_join[3], ctx->side_stream[3]));
      T9_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ev_join[3], 0));
   }
   return st;
}

static int md_kinetic(Context* ctx, double* ekin)
{
   const int nb = std::min(RED_MAX, grid_for(ctx->n, 256));
   k_md_kinetic<<<nb, 256, 0, ctx->stream>>>(ctx->n, ctx->md_v, ctx->md_minv, ctx->md_red, ctx->md_out,
      ctx->md_ticket);
   T9_CUDA(cudaGetLastError());
   double e;
   T9_CUDA(cudaMemcpyAsync(&e, ctx->md_out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   *ekin = e / EKCAL;  // kcal/mol
   return T9GB_OK;
}

}  // namespace t9gb

using namespace t9gb;

extern "C" int t9gb_md_init(t9gb_context* h, const double* xyz, const double* mass, const double* vel)
{
   if (!h || !xyz || !mass)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->have_topology)
      return T9GB_NOT_READY;
   const int n = ctx->n;
   std::vector<double> minv(n);
   for (int i = 0; i < n; ++i) {
      if (!(mass[i] > 0) || !std::isfinite(mass[i]))
         return T9GB_BAD_ARG;
      minv[i] = 1.0 / mass[i];
   }
   for (int i = 0; i < 3 * n; ++i)
      if (!std::isfinite(xyz[i]) || (vel && !std::isfinite(vel[i])))
         return T9GB_BAD_ARG;
   md_free(ctx);
   T9_CUDA(cudaMalloc(&ctx->md_x, sizeof(double) * 3 * n));
   T9_CUDA(cudaMalloc(&ctx->md_v, sizeof(double) * 3 * n));
   T9_CUDA(cudaMalloc(&ctx->md_minv, sizeof(double) * n));
   T9_CUDA(cudaMalloc(&ctx->md_g, sizeof(float) * 3 * n));
   T9_CUDA(cudaMalloc(&ctx->md_g2, sizeof(float) * 3 * n));
   T9_CUDA(cudaMalloc(&ctx->md_red, sizeof(double) * RED_MAX));
   T9_CUDA(cudaMalloc(&ctx->md_out, sizeof(double) * 2 + sizeof(int) * 2));
   ctx->md_ticket = reinterpret_cast<int*>(ctx->md_out + 2);
   T9_CUDA(cudaMemset(ctx->md_out, 0, sizeof(double) * 2 + sizeof(int) * 2));
   T9_CUDA(cudaMemcpy(ctx->md_x, xyz, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
   T9_CUDA(cudaMemcpy(ctx->md_minv, minv.data(), sizeof(double) * n, cudaMemcpyHostToDevice));
   if (vel)
      T9_CUDA(cudaMemcpy(ctx->md_v, vel, sizeof(double) * 3 * n, cudaMemcpyHostToDevice));
   else
      T9_CUDA(cudaMemset(ctx->md_v, 0, sizeof(double) * 3 * n));
   T9_CUDA(cudaDeviceSynchronize());
   // the force kernels' coordinates, the spatial order, and the first forces
   // (the integrator's KickOff)
   T9_CHECK(t9gb_set_xyz_host(h, xyz));
   if (!ctx->have_order)
      T9_CHECK(t9gb_nblist_build(h));
   T9_CHECK(md_forces(ctx, h));
   ctx->md_steps = ctx->md_iters = 0;
   ctx->md_ready = true;
   return T9GB_OK;
}

extern "C" int t9gb_md_run(t9gb_context* h, int nsteps, double dt, int thermostat, double kelvin, double tau,
   int nfree, unsigned long long seed, double* ekin_out, double* temp_out)
{
   if (!h || nsteps < 0 || !(dt > 0) || thermostat < 0 || thermostat > 1)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->md_ready)
      return T9GB_NOT_READY;
   const int n = ctx->n;
   if (nfree <= 0)
      nfree = 3 * n - 3;
   if (thermostat == 1 && (!(kelvin > 0) || !(tau > 0) || nfree < 2))
      return T9GB_BAD_ARG;
   if (thermostat == 1 && ctx->md_seed != seed) {
      ctx->md_rng.seed(seed);
      ctx->md_seed = seed;
   }
   const int nb = grid_for(3 * n, 256);
   const bool extra = ctx->use_vdw || ctx->nval > 0;
   if (thermostat == 1 && nsteps > 0) {
      // the run's thermostat variates, drawn in the reference's order (one
      // normal, then one chi-squared with nfree - 1 degrees, per step)
      std::vector<double> rs(2 * (size_t)nsteps);
      std::normal_distribution<double> gauss(0.0, 1.0);
      std::gamma_distribution<double> gam(0.5 * (nfree - 1), 2.0);
      for (int k = 0; k < nsteps; ++k) {
         rs[2 * k] = gauss(ctx->md_rng);
         rs[2 * k + 1] = gam(ctx->md_rng);
      }
      if (ctx->md_rs_cap < nsteps) {
         if (ctx->md_rs)
            T9_CUDA(cudaFree(ctx->md_rs));
         T9_CUDA(cudaMalloc(&ctx->md_rs, sizeof(double) * 2 * nsteps));
         ctx->md_rs_cap = nsteps;
      }
      T9_CUDA(cudaMemcpyAsync(ctx->md_rs, rs.data(), sizeof(double) * 2 * nsteps, cudaMemcpyHostToDevice,
         ctx->stream));
      T9_CUDA(cudaStreamSynchronize(ctx->stream));
   }
   for (int step = 0; step < nsteps; ++step) {
      k_md_kick<<<nb, 256, 0, ctx->stream>>>(n, 0.5 * dt, ctx->md_g, extra ? ctx->md_g2 : nullptr, ctx->md_minv,
         ctx->md_v);
      k_md_drift<<<nb, 256, 0, ctx->stream>>>(n, dt, ctx->md_v, ctx->md_x, ctx->xyz);
      T9_CUDA(cudaGetLastError());
      // a solve that fails to converge leaves no forces: the trajectory stops
      // there, as the reference's induce throws (src/cu/amoeba/pcg.cu:180-184)
      const int st = md_forces(ctx, h);
      if (st != T9GB_OK)
         return st;
      ctx->md_steps += 1;
      ctx->md_iters += ctx->last_iter;
      k_md_kick<<<nb, 256, 0, ctx->stream>>>(n, 0.5 * dt, ctx->md_g, extra ? ctx->md_g2 : nullptr, ctx->md_minv,
         ctx->md_v);
      T9_CUDA(cudaGetLastError());
      if (thermostat == 1) {
         // kinetic energy, factor and rescale on the device: no synchronisation
         const int kb = std::min(RED_MAX, grid_for(n, 256));
         k_md_kinetic<<<kb, 256, 0, ctx->stream>>>(n, ctx->md_v, ctx->md_minv, ctx->md_red, ctx->md_out,
            ctx->md_ticket);
         k_md_bussi<<<1, 1, 0, ctx->stream>>>(ctx->md_rs, step, std::exp(-dt / tau), kelvin, nfree, ctx->md_out);
         k_md_scale<<<nb, 256, 0, ctx->stream>>>(n, ctx->md_out + 1, ctx->md_v);
         T9_CUDA(cudaGetLastError());
      }
   }
   // the context's host coordinates follow the trajectory (t9gb_nblist_build
   // orders from them)
   if (ekin_out || temp_out) {
      double ek;
      T9_CHECK(md_kinetic(ctx, &ek));
      if (ekin_out)
         *ekin_out = ek;
      if (temp_out)
         *temp_out = 2.0 * ek / (nfree * GASCONST);
   }
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return T9GB_OK;
}

extern "C" int t9gb_md_state(t9gb_context* h, double* xyz, double* vel, float* grad_device)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->md_ready)
      return T9GB_NOT_READY;
   const int n = ctx->n;
   if (xyz)
      T9_CUDA(cudaMemcpyAsync(xyz, ctx->md_x, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
   if (vel)
      T9_CUDA(cudaMemcpyAsync(vel, ctx->md_v, sizeof(double) * 3 * n, cudaMemcpyDeviceToHost, ctx->stream));
   if (grad_device) {
      const bool extra = ctx->use_vdw || ctx->nval > 0;
      k_md_grad_total<<<grid_for(3 * n, 256), 256, 0, ctx->stream>>>(n, ctx->md_g, extra ? ctx->md_g2 : nullptr,
         grad_device);
      T9_CUDA(cudaGetLastError());
   }
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return T9GB_OK;
}

extern "C" int t9gb_md_positions_device(t9gb_context* h, float* xyz_device)
{
   if (!h || !xyz_device)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->md_ready)
      return T9GB_NOT_READY;
   // the drift kernel keeps the float copy of the trajectory in caller order
   T9_CUDA(cudaMemcpyAsync(xyz_device, ctx->xyz, sizeof(float) * 3 * ctx->n, cudaMemcpyDeviceToDevice,
      ctx->stream));
   return T9GB_OK;
}

extern "C" int t9gb_md_stats(t9gb_context* h, long long* steps, long long* pcg_iterations)
{
   if (!h)
      return T9GB_BAD_ARG;
   Context* ctx = &h->c;
   if (!ctx->md_ready)
      return T9GB_NOT_READY;
   if (steps)
      *steps = ctx->md_steps;
   if (pcg_iterations)
      *pcg_iterations = ctx->md_iters;
   return T9GB_OK;
}
