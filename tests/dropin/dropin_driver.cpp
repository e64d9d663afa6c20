// A Tinker9-style caller of the drop-in C++ entry points (t9gb_tinker.hpp):
// it sets the reference's module globals, binds a library context and calls
// tinker::induce / dfield / ufield / diagPrecond / sparsePrecondApply /
// empole / epolar / emplar the way the reference's ANALYZE driver does,
// then writes every result to a file for the test to compare with the
// C-ABI calls.  Test infrastructure only.
//
// usage: dropin_driver <input.bin> <output.bin>
//   input: t9gb_config (raw), int nexcl, frames int[n][4], pole double[n][10],
//          polarity/thole/pdamp double[n], excl_ik int[nexcl][2],
//          excl_scale double[nexcl][4], xyz double[n][3], probe double[n][3]
//   output (all little-endian, in order):
//          uind, uinp, udir, udirp float[n][3] from induce;
//          dfield d, p float[n][3]; ufield(probe, -probe) d, p float[n][3];
//          diagPrecond(probe, -probe) d, p; sparsePrecondApply(probe, -probe) d, p;
//          for empole, epolar, emplar: energy_em, energy_ep double, virial double[9],
//          gradient fixed u64 [3][n] (x, y, z rows);
//          int: 1 if induce with politer = 1 threw tinker::FatalError
#include <cuda_runtime_api.h>

#include <cstdio>
#include <cstring>
#include <vector>

#include "t9gb_tinker.hpp"

template <class T>
static void rd(FILE* f, T* p, size_t cnt)
{
   if (cnt && fread(p, sizeof(T), cnt, f) != cnt)
      throw tinker::FatalError("short input file");
}

template <class T>
static void wr(FILE* f, const T* p, size_t cnt)
{
   if (cnt && fwrite(p, sizeof(T), cnt, f) != cnt)
      throw tinker::FatalError("short write");
}

static void ck(cudaError_t e)
{
   if (e != cudaSuccess)
      throw tinker::FatalError(cudaGetErrorString(e));
}

template <class T>
static T* dev(size_t cnt)
{
   T* p = nullptr;
   ck(cudaMalloc((void**)&p, sizeof(T) * cnt));
   ck(cudaMemset(p, 0, sizeof(T) * cnt));
   return p;
}

template <class T>
static void out_dev(FILE* f, const T* d, size_t cnt)
{
   std::vector<T> h(cnt);
   ck(cudaDeviceSynchronize());
   ck(cudaMemcpy(h.data(), d, sizeof(T) * cnt, cudaMemcpyDeviceToHost));
   wr(f, h.data(), cnt);
}

static t9gb_context* make_ctx(const t9gb_config& cfg, const std::vector<int>& frames, const std::vector<double>& pole,
   const std::vector<double>& pol, const std::vector<double>& thl, const std::vector<double>& pdm, int nexcl,
   const std::vector<int>& eik, const std::vector<double>& esc)
{
   t9gb_context* ctx = nullptr;
   if (t9gb_create(&cfg, &ctx) != T9GB_OK)
      throw tinker::FatalError("t9gb_create failed");
   if (t9gb_set_topology(ctx, frames.data(), pole.data(), pol.data(), thl.data(), pdm.data(), nexcl, eik.data(),
          esc.data()) != T9GB_OK)
      throw tinker::FatalError("t9gb_set_topology failed");
   return ctx;
}

int main(int argc, char** argv)
{
   if (argc == 2 && std::strcmp(argv[1], "--link-check") == 0) {
      // resolves every drop-in symbol without touching a GPU
      void (*fns[])(int) = {tinker::empole, tinker::epolar, tinker::emplar, tinker::mpoleInit};
      std::printf("linked %zu term entry points, induce at %p\n", sizeof(fns) / sizeof(fns[0]),
         (void*)&tinker::induce);
      return 0;
   }
   if (argc != 3) {
      std::fprintf(stderr, "usage: %s input.bin output.bin | --link-check\n", argv[0]);
      return 2;
   }
   try {
      FILE* fi = std::fopen(argv[1], "rb");
      if (!fi)
         throw tinker::FatalError("cannot open input");
      t9gb_config cfg;
      rd(fi, &cfg, 1);
      int nexcl = 0;
      rd(fi, &nexcl, 1);
      const int n = cfg.n;
      std::vector<int> frames(4 * n), eik(2 * nexcl);
      std::vector<double> pole(10 * n), pol(n), thl(n), pdm(n), esc(4 * nexcl), xyz(3 * n), probe(3 * n);
      rd(fi, frames.data(), frames.size());
      rd(fi, pole.data(), pole.size());
      rd(fi, pol.data(), n);
      rd(fi, thl.data(), n);
      rd(fi, pdm.data(), n);
      rd(fi, eik.data(), eik.size());
      rd(fi, esc.data(), esc.size());
      rd(fi, xyz.data(), xyz.size());
      rd(fi, probe.data(), probe.size());
      std::fclose(fi);

      t9gb_context* ctx = make_ctx(cfg, frames, pole, pol, thl, pdm, nexcl, eik, esc);

      // the reference's module globals
      tinker::n = n;
      std::vector<float> hx(n), hy(n), hz(n);
      for (int i = 0; i < n; ++i) {
         hx[i] = (float)xyz[3 * i];
         hy[i] = (float)xyz[3 * i + 1];
         hz[i] = (float)xyz[3 * i + 2];
      }
      tinker::x = dev<float>(n);
      tinker::y = dev<float>(n);
      tinker::z = dev<float>(n);
      ck(cudaMemcpy(tinker::x, hx.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
      ck(cudaMemcpy(tinker::y, hy.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
      ck(cudaMemcpy(tinker::z, hz.data(), sizeof(float) * n, cudaMemcpyHostToDevice));
      using v3 = tinker::real(*)[3];
      tinker::uind = (v3)dev<float>(3 * n);
      tinker::uinp = (v3)dev<float>(3 * n);
      tinker::udir = (v3)dev<float>(3 * n);
      tinker::udirp = (v3)dev<float>(3 * n);
      tinker::demx = dev<tinker::grad_prec>(n);
      tinker::demy = dev<tinker::grad_prec>(n);
      tinker::demz = dev<tinker::grad_prec>(n);
      tinker::depx = dev<tinker::grad_prec>(n);
      tinker::depy = dev<tinker::grad_prec>(n);
      tinker::depz = dev<tinker::grad_prec>(n);
      tinker::rc_flag = tinker::calc::xyz | tinker::calc::vmask;
      tinker::t9gbBind(ctx);

      FILE* fo = std::fopen(argv[2], "wb");
      if (!fo)
         throw tinker::FatalError("cannot open output");

      // ANALYZE order: rotate the multipoles, then the solve
      tinker::mpoleInit(tinker::calc::v1);
      tinker::induce(tinker::uind, tinker::uinp);
      out_dev(fo, &tinker::uind[0][0], 3 * n);
      out_dev(fo, &tinker::uinp[0][0], 3 * n);
      out_dev(fo, &tinker::udir[0][0], 3 * n);
      out_dev(fo, &tinker::udirp[0][0], 3 * n);

      v3 f = (v3)dev<float>(3 * n), fp = (v3)dev<float>(3 * n);
      v3 a = (v3)dev<float>(3 * n), b = (v3)dev<float>(3 * n);
      std::vector<float> pa(3 * n), pb(3 * n);
      for (int i = 0; i < 3 * n; ++i) {
         pa[i] = (float)probe[i];
         pb[i] = (float)-probe[i];
      }
      ck(cudaMemcpy(a, pa.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
      ck(cudaMemcpy(b, pb.data(), sizeof(float) * 3 * n, cudaMemcpyHostToDevice));
      tinker::dfield(f, fp);
      out_dev(fo, &f[0][0], 3 * n);
      out_dev(fo, &fp[0][0], 3 * n);
      tinker::ufield(a, b, f, fp);
      out_dev(fo, &f[0][0], 3 * n);
      out_dev(fo, &fp[0][0], 3 * n);
      tinker::diagPrecond(a, b, f, fp);
      out_dev(fo, &f[0][0], 3 * n);
      out_dev(fo, &fp[0][0], 3 * n);
      tinker::sparsePrecondApply(a, b, f, fp);
      out_dev(fo, &f[0][0], 3 * n);
      out_dev(fo, &fp[0][0], 3 * n);

      void (*terms[3])(int) = {tinker::empole, tinker::epolar, tinker::emplar};
      for (int t = 0; t < 3; ++t) {
         terms[t](tinker::calc::v1);
         const bool polar = t == 1;
         wr(fo, &tinker::energy_em, 1);
         wr(fo, &tinker::energy_ep, 1);
         wr(fo, polar ? tinker::virial_ep : tinker::virial_em, 9);
         out_dev(fo, polar ? tinker::depx : tinker::demx, n);
         out_dev(fo, polar ? tinker::depy : tinker::demy, n);
         out_dev(fo, polar ? tinker::depz : tinker::demz, n);
      }

      // the reference's non-convergence error: one iteration allowed
      t9gb_config c1 = cfg;
      c1.politer = 1;
      t9gb_context* ctx1 = make_ctx(c1, frames, pole, pol, thl, pdm, nexcl, eik, esc);
      tinker::t9gbBind(ctx1);
      int threw = 0;
      try {
         tinker::mpoleInit(tinker::calc::v0);
         tinker::induce(tinker::uind, tinker::uinp);
      } catch (const tinker::FatalError& e) {
         std::printf("FatalError: %s\n", e.what());
         threw = 1;
      }
      wr(fo, &threw, 1);
      std::fclose(fo);
      tinker::t9gbUnbind();
      t9gb_destroy(ctx1);
      t9gb_destroy(ctx);
   } catch (const tinker::FatalError& e) {
      std::fprintf(stderr, "FatalError: %s\n", e.what());
      return 1;
   }
   return 0;
}
