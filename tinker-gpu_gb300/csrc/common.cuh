// Shared definitions of the GB300 polarization library: the context that owns
// every device buffer, fixed-point helpers, the Hastings erfc, and the
// per-kernel event profiler.
#pragma once
#include <cuda_bf16.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <cstdint>
#include <functional>
#include <random>
#include <string>
#include <vector>

#include "../../include/t9gb.h"

namespace t9gb {

constexpr int WARP = 32;
constexpr int BSORDER = 5;
constexpr int GROUP = 16;  // lanes per atom in the real-space kernels

// The PME grid accumulates in signed 64-bit fixed point with 40 fractional
// bits: order-independent (bit-reproducible) sums, range +-8.4e6,
// resolution 9.1e-13.
constexpr double FX_SCALE = 1099511627776.0;  // 2^40
constexpr double FX_INV = 1.0 / 1099511627776.0;

// Conversions in 32-bit arithmetic (64-bit conversions and FP64 are slow
// paths on this GPU).  to_fx: y = v 2^8 = hi + frac with hi = floor(y) and
// frac in [0, 1) exact, so hi 2^32 + rn(frac 2^32) = rn(v 2^40), the value
// a direct float -> int64 conversion gives (|v| < 2^23).  from_fx:
// v 2^-40 = hi 2^-8 + lo 2^-40 for v = hi 2^32 + lo, within one rounding of
// the correctly rounded float.
__device__ __forceinline__ long long to_fx(float v)
{
   const float y = v * 256.0f;
   const int hi = __float2int_rd(y);
   const unsigned lo = __float2uint_rn((y - (float)hi) * 4294967296.0f);
   return (long long)(((unsigned long long)(long long)hi << 32) + lo);
}
__device__ __forceinline__ float from_fx(long long v)
{
   const int hi = (int)(v >> 32);
   const unsigned lo = (unsigned)(v & 0xffffffffll);
   return fmaf(__uint2float_rn(lo), 9.094947017729282e-13f, __int2float_rn(hi) * 0.00390625f);
}

// Complementary error function, Hastings' rational approximation (C. Hastings,
// Approximations for Digital Computers, Princeton 1955, p. 167; Abramowitz &
// Stegun 7.1.26), sharing exp(-x^2) with the caller; the reference's float
// build uses the same approximation (include/math/libfunc.h:12-28).
__device__ __forceinline__ float erfc_hastings(float x, float expmx2)
{
   float t = __frcp_rn(1.0f + 0.3275911f * x);
   return (0.254829592f + (-0.284496736f + (1.421413741f + (-1.453152027f + 1.061405429f * t) * t) * t) * t) * t
      * expmx2;
}

__device__ __forceinline__ float image1(float d, float l, float linv) { return d - l * rintf(d * linv); }

struct PmeGrid {
   int n1 = 0, n2 = 0, n3 = 0;
   bool own_fft = false;      // power-of-two grid: the library's fused FFT path
   bool own_fft_ok = false;   // the grid qualifies
   cufftHandle plan = 0, plan2 = 0;
   float2* qgrid = nullptr;   // complex grid [n3][n2][n1]
   long long* qfx = nullptr;  // fixed-point accumulation grid [n3][n2][n1], one word per point
   float2* qgrid2 = nullptr;  // the second grid pair (induced-dipole reciprocal forces)
   long long* qfx2 = nullptr;
   float* infl = nullptr;     // influence function [n3][n2][n1]
   float2* qstash = nullptr;  // transformed permanent grid kept for the virial cross terms
   bool packed = false;       // the fixed-point grid holds packed d / p dipole values
   int pack_shift = 24;       // their 32-bit fixed-point scale 2^pack_shift (16 after a range fallback)
   bool probe = false;        // spreads of the learned guess's residual: their own range flag
   int fft_cl = 0;            // fused transform: CTAs per z plane (a thread-block cluster), 0: one CTA
   int* fft_err = nullptr;    // device flag: a staged slab copy of a plane pass did not complete in time
};

// Per-kernel event timing (tracing): categories of timed launches.
enum ProfCat {
   P_DFIELD_REAL = 0,
   P_UFIELD_REAL,
   P_PRECOND,
   P_SPREAD_MPOLE,
   P_SPREAD_UIND,
   P_FFT_CONV,
   P_GATHER_MPOLE,
   P_GATHER_UIND,
   P_VECTOR,
   P_NBLIST,
   P_NCAT
};

struct Profiler {
   bool on = false;
   std::vector<cudaEvent_t> ev;  // pairs
   std::vector<int> cat;
   int used = 0;
   double ms[P_NCAT] = {0};
   long long cnt[P_NCAT] = {0};
};

// Learned-guess network: 32 -> 64 -> 64 -> 3 (output padded to 8 columns)
constexpr int MLP_IN = 32, MLP_HID = 64, MLP_OUT = 3, MLP_OUT_PAD = 8;
constexpr int MLP_NPARAM = MLP_IN * MLP_HID + MLP_HID + MLP_HID * MLP_HID + MLP_HID + MLP_HID * MLP_OUT_PAD + MLP_OUT_PAD;

struct MlpState {
   int max_rows = 0;
   int* step = nullptr; // AdamW steps taken (device, so graphs replay it)
   int nsplit = 64;     // batch splits of the weight-gradient GEMMs
   float* w = nullptr;  // FP32 master parameters
   float* g = nullptr;  // gradient
   float* m = nullptr;  // AdamW moments
   float* v = nullptr;
   unsigned char* mask = nullptr;
   int* wb_index = nullptr;
   __nv_bfloat16* wb = nullptr;  // BF16 weights used by the GEMMs
   __nv_bfloat16* x = nullptr;   // [rows][32] inputs
   float* z1 = nullptr;          // [rows][64] pre-activations
   float* z2 = nullptr;
   __nv_bfloat16* h1 = nullptr;  // [rows][64] activations
   __nv_bfloat16* h2 = nullptr;
   float* c = nullptr;           // [rows][64] GEMM output scratch
   float* y = nullptr;           // [rows][8] outputs
   float* t = nullptr;           // [rows][3] targets
   __nv_bfloat16* dy = nullptr;  // [rows][8]
   float* dyf = nullptr;
   __nv_bfloat16* dz = nullptr;  // [rows][64]
   float* dzf = nullptr;
   double* err = nullptr;        // [rows] squared error
   double* loss = nullptr;
   float* split = nullptr;       // split-K / column-sum partials
   float* gpart = nullptr;       // [rows / 128][MLP_NPARAM] per-CTA gradients (tcgen05 training pass)
   int* ticket = nullptr;        // blocks done in the gradient sum (reset by the last)
   int sms = 1;                  // multiprocessors: CTAs of the training pass
};

struct Context {
   t9gb_config cfg;
   Profiler prof;
   MlpState mlp;
   int n = 0;
   int npad = 0;  // n rounded up to 32
   int dev = 0;
   cudaStream_t stream = nullptr;
   bool own_stream = false;
   std::string last_error;

   // topology, caller atom order
   int4* frames = nullptr;  // zaxis, xaxis, yaxis (1-based signed), kind
   float* pole = nullptr;   // [n][10] local frame
   std::vector<double> h_polarity, h_thole, h_pdamp;
   // per-type-pair Thole table (reference jpolar / thlval): when set, the
   // thole slot of every row holds the atom's polarization type instead
   std::vector<int> h_ptype;
   float* thl = nullptr;  // [nthl][nthl], device
   int nthl = 0;
   // uniform external field (reference extfld::texfld), e/A^2: device copy
   // read by the permanent-field kernel, host copy for the force path
   float* exfld = nullptr;  // [4], device
   float h_exfld[4] = {0.f, 0.f, 0.f, 0.f};
   bool use_exfld = false;
   std::vector<int> h_excl_ik;
   std::vector<double> h_excl_scale;

   // buffered 14-7 van der Waals (t9gb_set_vdw): per-type-pair radius and
   // well depth, reduction toward a parent atom, scaled pairs, taper / cutoff
   bool use_vdw = false;
   int nvt = 0;
   double vdw_taper = 0, vdw_off = 0;
   std::vector<int> h_vtype, h_vparent;
   std::vector<double> h_vred;
   std::vector<int> h_vexcl_ik;
   std::vector<double> h_vexcl_scale;
   float2* vtab = nullptr;     // [nvt][nvt] (radmin, epsilon), device
   int* vtype = nullptr;       // [n]
   int* vparent = nullptr;     // [n]
   float* vred = nullptr;      // [n]
   int* vch_start = nullptr;   // [n + 1] children (atoms reduced toward this one)
   int* vch = nullptr;
   float4* vpos = nullptr;     // [npad] reduced sites, sorted; w = type (int bits)
   float* fvdw = nullptr;      // [npad][3] dE/dx of each reduced site
   double* e_vdw = nullptr;    // [npad] van der Waals energy per site
   float* sp_v = nullptr;      // [nsp] van der Waals scale of each scaled pair

   // bond / angle / Urey-Bradley terms (t9gb_set_valence), caller order
   int nval = 0;
   double val_glob[8] = {0, 0, 0, 0, 0, 0, 0, 0};  // bond c/q, angle c/q/p/s, Urey c/q
   int4* val_idx = nullptr;    // [nval] (a, b, c, kind)
   float2* val_par = nullptr;  // [nval] (force constant, ideal)
   float* val_g = nullptr;     // [nval][3][3] gradient slots
   double* val_e = nullptr;    // [nval]
   float* val_w = nullptr;     // [9][nval] virial rows
   int* val_start = nullptr;   // [n + 1] per-atom slot lists
   int* val_ent = nullptr;
   double* val_sum = nullptr;  // [10]

   // molecular dynamics state (t9gb_md_init / t9gb_md_run), caller order
   double* md_x = nullptr;     // [n][3] positions, FP64
   double* md_v = nullptr;     // [n][3] velocities, A/ps
   double* md_minv = nullptr;  // [n] 1 / mass
   float* md_g = nullptr;      // [n][3] total gradient at md_x
   float* md_g2 = nullptr;     // [n][3] its van der Waals + valence part
   double* md_red = nullptr;   // kinetic-energy partials
   double* md_out = nullptr;   // [2] + ticket
   int* md_ticket = nullptr;
   bool md_ready = false;
   std::mt19937_64 md_rng;     // Bussi thermostat variates (host)
   double* md_rs = nullptr;    // [2][nsteps] variates of the current run
   int md_rs_cap = 0;
   unsigned long long md_seed = ~0ull;
   long long md_steps = 0, md_iters = 0;  // since t9gb_md_init

   // coordinates, caller order
   float* xyz = nullptr;       // [n][3]
   std::vector<double> h_xyz;  // host copy for the ordering, refreshed by t9gb_nblist_build
   float* h_in = nullptr;      // pinned staging of host coordinates
   cudaEvent_t ev_in = nullptr; // its last copy to the device
   cudaEvent_t ev_solved = nullptr;  // the induce graph and its status copies (work queued after it runs on)
   bool ev_in_pending = false;
   bool have_xyz = false;
   bool have_topology = false;
   bool have_order = false;

   // sorted layout: the internal order of every hot-path array
   int* perm = nullptr;   // slot -> atom (-1 for padding)
   int* iperm = nullptr;  // atom -> slot
   std::vector<int> h_perm, h_iperm;
   float4* spos = nullptr;   // [npad]
   float* spolar = nullptr;  // [npad] polarizability (0 on padding)
   float* spolinv = nullptr; // [npad] 1/max(alpha, 1e-16)
   float2* sdamp = nullptr;  // [npad] pdamp, thole
   float* srpole = nullptr;  // [npad][12] global-frame multipoles, thole, polarizability
   float* sframe = nullptr;  // [npad][9] local multipole frame (rows: x, y, z axes)

   // scaled partners of every slot, both directions (CSR over slots)
   int* sp_start = nullptr;  // [npad + 1]
   int* sp_j = nullptr;      // partner slot
   float4* sp_sc = nullptr;  // m, d, p, u
   int nsp = 0;

   // per-step neighbour list (exact cutoff, scaled partners excluded)
   float list_cut = 0;
   int nbr_cap = 0;
   int* nbr = nullptr;       // [npad][nbr_cap]
   int* nnbr = nullptr;      // [npad]
   // per-step sub-lists of nbr (same order): pairs within the cutoff and
   // within the preconditioner cutoff
   int* nbrc = nullptr;
   int* nnbrc = nullptr;
   int* nbrp = nullptr;
   int* nnbrp = nullptr;
   // staged field / preconditioner kernels (t9gb_pair_staging): per 32-slot
   // block the j-blocks its sub-list entries fall in (ascending, at most
   // STAGE_JB_CAP; jbn > cap means the block reads rows from global memory),
   // and every sub-list entry as a local index (j-block position x 32 +
   // slot within the block)
   int* jbl = nullptr;               // [npad / 32][STAGE_JB_CAP]
   int* jbn = nullptr;               // [npad / 32]
   unsigned short* nbrc_l = nullptr; // [npad][nbr_cap]
   unsigned short* nbrp_l = nullptr; // [npad][nbr_cap]
   bool pair_staged = false;         // t9gb_pair_staging
   bool mlp_tc = true;               // learned guess: forward pass on tcgen05 (t9gb_learn_tensor_path)
   int* copy_err = nullptr;          // device flag: a staging copy did not complete in time
   int* nbr_over = nullptr;  // device max count seen (overflow check)
   int* h_over = nullptr;    // pinned mirror
   int pair_lanes = 8;            // lanes per atom in the field kernels
   int pcg_fuse = 121;            // t9gb_set_pcg_fusion (bit 4: programmatic dependent launch, bits 5-6: gather and stream layout)
   int force_lanes = 4;           // lanes per atom in the real-space force kernel
   bool list_stale = true;        // positions changed since the last list check
   bool list_need_build = true;   // no valid list for the current order / capacity
   float4* sref = nullptr;        // [npad] positions at the last list build
   int* lflag = nullptr;          // device: rebuild requested / an atom moved too far
   int* h_lflag = nullptr;        // pinned mirror
   bool use_cells = false;
   int nc[3] = {0, 0, 0};
   int ncell = 0;
   int* cell_count = nullptr;
   int* cell_start = nullptr;  // [ncell + 1]
   int* cell_atoms = nullptr;  // [npad]
   int* atom_cell = nullptr;   // [npad]

   // PME
   PmeGrid pme;

   // fields and PCG work, all sorted rows of 8 floats: d xyz, p xyz, thole,
   // polarizability (32-byte rows; components 6-7 are set once per order)
   float* rcp6 = nullptr;   // reciprocal + self field
   float* fld6 = nullptr;   // total field of the last dfield/ufield
   float* udir = nullptr;
   float* efield = nullptr;
   float* uind = nullptr;
   float* rsd = nullptr;
   float* zrsd = nullptr;
   float* conj = nullptr;
   float* vec = nullptr;
   float* tmp6 = nullptr;
   double* e_atom = nullptr; // [3][npad] per-atom energy terms (real, recip, self)
   double* red = nullptr;   // reduction partials [RED_SLOTS][RED_MAX]
   double* scal = nullptr;  // device scalars
   int* status = nullptr;   // device status words
   int* h_status = nullptr; // pinned mirrors
   double* h_scal = nullptr;

   // predictor ring (ASPC 16 / Gear 6 frames), sorted [depth][npad][8]; the
   // ring count is device state
   float* aspc_hist = nullptr;
   // learned extrapolation of the ASPC ring (t9gb_learn_extrapolation)
   int lx_k = 0;                  // ring frames of the fit, 0: off
   double* lx_ab = nullptr;       // normal equations [8][8] + [8]
   float* lx_part = nullptr;      // per-block partial sums
   float* lx_coef_buf = nullptr;  // ring coefficients by frame age [16]
   float* lx_coef = nullptr;      // lx_coef_buf while on, else null
   int* lx_ticket = nullptr;      // last-block ticket of the fit
   cudaStream_t lx_stream = nullptr;  // the fit runs here, after the solve's graph
   cudaEvent_t ev_lx_fork = nullptr, ev_lx_done = nullptr;
   bool lx_pending = false;       // a fit is queued that the next solve waits for

   // learned initial guess (learn.cu)
   int learn_mode = 0;          // bit 0: train after each solve, bit 1: start from the learned guess
   unsigned learn_seed = 1;
   float learn_lr = 1e-3f, learn_wd = 1e-2f;
   float* xf = nullptr;         // [2 npad][32] raw features, d rows then p rows
   float* fstat = nullptr;      // feature mean[32], 1/std[32], target scale
   float* hout = nullptr;       // [6 n] host-copy staging

   // forces (force.cu): per-slot real / reciprocal (permanent grid,
   // dipole grid) forces and torque fields, frame forces by role, and the
   // reverse frame map (slot j -> (slot i, role) entries)
   float *freal = nullptr, *frecp = nullptr, *frecu = nullptr;
   float *treal = nullptr, *trecp = nullptr, *trecu = nullptr;
   float* fbuf = nullptr;
   float* wvir = nullptr;  // [27][npad] virial rows: real, frame, reciprocal
   double* vsum = nullptr; // their sums
   double* sum_part = nullptr; // [SUM_ROWS_MAX][SUM_PARTS] partials of the fixed-order row sums
   int *rev_start = nullptr, *rev_ent = nullptr;
   std::vector<int> h_frames;  // [n][4] caller order
   // start policy (host): compare the plain and the learned start every
   // learn_probe solves; in between reuse the last comparison's result
   int learn_probe = 1;
   int learn_since_probe = 1 << 30;
   int learn_last_choice = 0;
   int learn_variant = 0;       // start variant of the last solve
   bool learn_ring_full = false;

   // whole-induce CUDA graph
   bool use_graph = true;
   cudaGraphExec_t graph_exec[4] = {nullptr, nullptr, nullptr, nullptr};  // per start variant (pcg.cu)
   cudaStream_t cap_stream = nullptr;
   // t9gb_induce_host: enqueue the caller-order dipole copy before the
   // solve's one synchronisation
   bool stage_out = false;
   float* out_d = nullptr;  // t9gb_induce's device outputs, written before the solve's synchronisation
   float* out_p = nullptr;
   // work queued behind the induce graph before the solve's synchronisation
   // (the MD step's forces); after_done: it ran; induce_redone: the solve was
   // repeated after it ran (a list or range retry), so it used a discarded solve
   const std::function<int()>* after_launch = nullptr;
   bool after_done = false;
   bool induce_redone = false;
   // second streams for the reciprocal grid half of a field evaluation, run
   // beside the real-space pair kernel (fork / join by events).  A stream
   // that joined a graph capture stays in it until that capture ends, so the
   // WHILE-body capture (on cap_stream) has its own side stream: [1] there,
   // [0] everywhere else.
   // side streams: [0] eager forks, [1] forks inside a graph capture, [2] the
   // second reciprocal half of the forces, [3] the MD step's van der Waals
   // and valence terms beside the electrostatic forces
   cudaStream_t side_stream[4] = {nullptr, nullptr, nullptr, nullptr};
   cudaEvent_t ev_fork[4] = {nullptr, nullptr, nullptr, nullptr}, ev_join[4] = {nullptr, nullptr, nullptr, nullptr};

   // last induce statistics
   int last_iter = 0;
   double last_eps = 0;
   int last_status = 0;

   // pinned staging for host entry points
   float* h_stage = nullptr;
   size_t h_stage_bytes = 0;
};

// reductions: up to RED_MAX block partials per slot
// Largest separation between the two reduced van der Waals sites of a pair
// and their atoms' separation that the stored list allows for (each site lies
// (1 - red) of a bond from its atom: 0.09 A for AMOEBA water hydrogens).
constexpr double VDW_SITE_MARGIN = 0.25;
// j-blocks a 32-slot block stages into shared memory (48 of 1.5 KB: 72 KB,
// three blocks per SM); water blocks need 39 on average, 45 at most at a
// 7 A cutoff
constexpr int STAGE_JB_CAP = 48;

// energy / virial row sums: at most SUM_ROWS_MAX rows per launch, each
// split over SUM_PARTS blocks
constexpr int SUM_ROWS_MAX = 32, SUM_PARTS = 8;
constexpr int RED_MAX = 2048;
constexpr int RED_SLOTS = 8;

#define T9_CUDA(call)                                                                                                  \
   do {                                                                                                                \
      cudaError_t err_ = (call);                                                                                       \
      if (err_ != cudaSuccess) {                                                                                       \
         ctx->last_error = std::string(#call) + ": " + cudaGetErrorString(err_);                                       \
         return T9GB_CUDA_ERR;                                                                                         \
      }                                                                                                                \
   } while (0)

#define T9_CHECK(expr)                                                                                                 \
   do {                                                                                                                \
      int rc_ = (expr);                                                                                                \
      if (rc_ != T9GB_OK)                                                                                              \
         return rc_;                                                                                                   \
   } while (0)

inline int grid_for(long long n, int block) { return (int)((n + block - 1) / block); }

// Programmatic dependent launch.  A kernel launched with launch_k(pdl =
// true) may be scheduled while the kernel before it on the stream drains;
// every such kernel calls pdl_wait() first, which returns once that kernel
// has completed and its memory is visible (a no-op for a plain launch).
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
// lets the next kernel on the stream launch (its pdl_wait still waits for
// this grid's completion); issued once a thread's main loop is done
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

template <typename... KArgs, typename... Args>
inline cudaError_t launch_k(bool pdl, void (*kernel)(KArgs...), dim3 grid, dim3 block, size_t smem, cudaStream_t st,
   Args... args)
{
   if (!pdl) {
      kernel<<<grid, block, smem, st>>>(static_cast<KArgs>(args)...);
      return cudaGetLastError();
   }
   cudaLaunchConfig_t cfg = {};
   cfg.gridDim = grid;
   cfg.blockDim = block;
   cfg.dynamicSmemBytes = smem;
   cfg.stream = st;
   cudaLaunchAttribute at[1];
   at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
   at[0].val.programmaticStreamSerializationAllowed = 1;
   cfg.attrs = at;
   cfg.numAttrs = 1;
   return cudaLaunchKernelEx(&cfg, kernel, static_cast<KArgs>(args)...);
}

// programmatic dependent launch for the kernels of the PCG loop (fusion bit
// 4), outside the per-kernel timing mode
inline bool use_pdl(const Context* ctx) { return (ctx->pcg_fuse & 16) && !ctx->prof.on; }

// Bounded wait on phase `phase` (parity) of an mbarrier in shared memory
// (shared::cta address); false when the limit (about a second of polling)
// ran out, so a copy that never completes cannot hang the kernel.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned bar, unsigned phase)
{
   for (int it = 0; it < (1 << 20); ++it) {
      unsigned ok;
      asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
                   : "=r"(ok)
                   : "r"(bar), "r"(phase)
                   : "memory");
      if (ok)
         return true;
   }
   return false;
}

__device__ __forceinline__ void mbar_init(unsigned bar, unsigned count)
{
   asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(bar), "r"(count) : "memory");
   asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_expect_tx(unsigned bar, unsigned bytes)
{
   asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(bytes) : "memory");
}

// bulk asynchronous copy global -> this CTA's shared memory (16-byte aligned
// addresses, size a multiple of 16), completing on the mbarrier
__device__ __forceinline__ void bulk_g2s(unsigned dst, const void* src, unsigned bytes, unsigned bar)
{
   asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                "l"(src), "r"(bytes), "r"(bar)
                : "memory");
}

// timed launch bracket; a no-op unless profiling is on
inline void prof_begin(Context* ctx, int cat)
{
   Profiler& p = ctx->prof;
   if (!p.on || p.used + 1 >= (int)p.cat.size())
      return;
   cudaEventRecord(p.ev[2 * p.used], ctx->stream);
   p.cat[p.used] = cat;
}
inline void prof_end(Context* ctx)
{
   Profiler& p = ctx->prof;
   if (!p.on || p.used + 1 >= (int)p.cat.size())
      return;
   cudaEventRecord(p.ev[2 * p.used + 1], ctx->stream);
   p.used++;
}
// accumulate recorded pairs (call after the stream is synchronised)
inline void prof_collect(Context* ctx)
{
   Profiler& p = ctx->prof;
   for (int i = 0; i < p.used; ++i) {
      float ms = 0;
      if (cudaEventElapsedTime(&ms, p.ev[2 * i], p.ev[2 * i + 1]) == cudaSuccess) {
         p.ms[p.cat[i]] += ms;
         p.cnt[p.cat[i]] += 1;
      }
   }
   p.used = 0;
}

// ---- entry points implemented across the translation units ----
int order_build(Context* ctx);  // host: spatial order, scaled partners
int list_update(Context* ctx);  // device: exact neighbour list
int ensure_list(Context* ctx);  // list_update when the coordinates changed
int check_list_overflow(Context* ctx, int* redo);
int lx_config(Context* ctx, int order);   // pcg.cu
int lx_state(Context* ctx, int* fits, int* rejected, float* coef16);  // pcg.cu
int lx_wait(Context* ctx);                // pcg.cu
int alloc_lists(Context* ctx, int cap);          // nbr, nbrc, nbrp with row capacity cap
int pair_staging_setup();                         // pair.cu: shared-memory limits of the staged kernels
int mlp_tc_setup();                               // mlp.cu: shared-memory limit of the tcgen05 forward
int launch_list_filter(Context* ctx);             // pair.cu  // after a sync; redo = 1: grown, repeat
// The fused kernels of a CG iteration: the sparse preconditioner with the
// r.z / r.r sums and the CG scalars (pair.cu), and the mutual-field gather
// with Ap = p/alpha - field, p.Ap and the step length (pme.cu).
struct PcgDots {
   float* conj;  // init: the first search direction p = z
   double* red;
   double* scal;
   int* state;
   int init, n;
   double debye, poleps;
   int politer, miniter;
   cudaGraphConditionalHandle handle;
   int use_handle;
};
struct PcgAp {
   const float* zrsd;    // z: p = z + b p_old
   float* conj;          // p_old in, p out
   const float* polinv;  // 1/alpha per slot
   float* vec;           // Ap out
   double* red;
   double* scal;
   int* state;
};
int launch_precond_sparse_dots(Context* ctx, const float* r6, float* z6, const PcgDots& D);
int launch_ufield_real_dir(Context* ctx, const float* p6, const float* z6, const double* scal, float* out6);
int launch_ufield_recip_grid_dir(Context* ctx, const float* p6, const float* z6, const double* scal);
int launch_ufield_recip_gather_ap(Context* ctx, float* out6, const PcgAp& P);
int launch_ufield_recip_gather_dir(Context* ctx, float* out6, const PcgAp& P);
// the same on the second grid (and FFT plan)
int launch_ufield_recip_grid_alt(Context* ctx, const float* u6);
int launch_ufield_recip_gather_alt(Context* ctx, const float* u6, float* out6);
int scatter_positions(Context* ctx);
// t9gb_emplar(grad) with `beside` called once the dipoles are solved and the
// list is current, before the electrostatic forces are launched
int emplar_grad_beside(Context* ctx, float* grad, const std::function<int()>& beside,
   const std::function<int()>& reset);
// side stream of the current capture level, and the fork / join of work on
// it with the main stream (events, no host synchronisation)
int side_index(const Context* ctx);
int recip_fork(Context* ctx, int k);
int recip_join(Context* ctx, int k);
int rotpole_sorted(Context* ctx);
int reset_predictor(Context* ctx);
// ring depth of the dipole predictor: ASPC 16, Gear 6, none 0
// (maxualt, src/amoeba/epolar.cpp:446-470)
static inline int pred_depth(const t9gb_config& c) { return c.predictor == 1 ? 16 : c.predictor == 2 ? 6 : 0; }
int fill_row_padding(Context* ctx);
int pme_setup(Context* ctx);
void pme_free(Context* ctx);

// real space (pair.cu): out6 = base6 (may be null) + real-space field
int launch_dfield_real(Context* ctx, const float* base6, float* out6);
int launch_ufield_real(Context* ctx, const float* u6, const float* base6, float* out6);
int launch_precond_sparse(Context* ctx, const float* r6, float* z6);

// reciprocal space (pme.cu): out6 = recip + self field (plain store)
int launch_dfield_recip(Context* ctx, float* out6);
int launch_ufield_recip(Context* ctx, const float* u6, float* out6);
int launch_dfield_recip_grid(Context* ctx);
int launch_dfield_recip_gather(Context* ctx, float* out6, bool acc);
int launch_ufield_recip_grid(Context* ctx, const float* u6);
int launch_ufield_recip_gather(Context* ctx, const float* u6, float* out6, bool acc);

// energies: per-atom FP64 terms (pair.cu real space, pme.cu recip + self)
int launch_empole_real(Context* ctx, double* e_atom);
int launch_empole_recip(Context* ctx, double* e_atom);

// learned-guess network (mlp.cu)
int mlp_alloc(Context* ctx, int max_rows, unsigned seed);
void mlp_free(Context* ctx);
int mlp_set_weights(Context* ctx, const float* w_host);
int mlp_get_weights(Context* ctx, float* w_host);
int mlp_forward(Context* ctx, int rows);
int mlp_backward(Context* ctx, int rows, const float* rowpol, int npad);
// tcgen05 path: recomputed forward, loss, gradient and AdamW step in two
// launches; scal (may be null) takes the summed squared error x loss_norm
int mlp_train_step_tc(Context* ctx, int rows, const float* rowpol, int npad, float lr, float wd, double* scal,
   double loss_norm);
int mlp_adamw(Context* ctx, float lr, float wd);
// learned guess (learn.cu)
int launch_learn_features(Context* ctx, const float* e8, const float* u8, float* xf, const float* fstat,
   __nv_bfloat16* xn);  // pair.cu
// forces (force.cu, pme.cu)
int force_setup(Context* ctx);
void force_free(Context* ctx);
int frame_map_build(Context* ctx);
int elec_forces(Context* ctx, bool mpole, bool polar, float* grad, bool vir);
// external-field multipole terms after the pair / reciprocal kernels:
// energy into the one-body block of e_atom, forces, torque field, virial rows
int launch_extfield_mpole(Context* ctx, bool forces, bool vir);
int launch_force_recip(Context* ctx, bool mpole, bool polar, float* wrec);
int launch_force_recip_perm(Context* ctx, bool mpole, bool polar, float* wrec);
int launch_force_recip_uind(Context* ctx, float* wrec, bool alt);
int induce_sorted(Context* ctx);
int learn_setup(Context* ctx);
void learn_free(Context* ctx);
int learn_reset(Context* ctx, unsigned seed);
int learn_forward(Context* ctx, bool need_y);
int learn_guess(Context* ctx, float* ug8, int set_choice);
void drop_graphs(Context* ctx);  // pcg.cu
// energy.cu: fixed-order sums of per-slot rows (nrows <= 8 FP64 rows; nblocks
// <= 3 blocks of 9 FP32 virial rows, summed and symmetrised)
int sum_rows_d(Context* ctx, const double* rows, int nrows, double* out);
int sum_rows_virial(Context* ctx, const float* rows, int nblocks, double* virial);
// vdw.cu: reduced sites, pair kernel and per-atom gather (grad: dE/dx added
// to or stored in grad when not null); energy rows in e_atom[2 npad ..)
int vdw_forces(Context* ctx, float* grad, bool add, bool vir, double* energy);
void vdw_release(Context* ctx);
// valence.cu: bond / angle / Urey-Bradley gradient (into or added to grad),
// then their energy and virial sums
int valence_forces(Context* ctx, float* grad, bool add, bool vir);
int valence_sums(Context* ctx, double* energy, double* virial);
void valence_release(Context* ctx);
void md_release(Context* ctx);  // md.cu
int learn_pick(Context* ctx, const float* ug8, const float* fld8);
int learn_train(Context* ctx);
int learn_features_out(Context* ctx, float* out_dev);

// permutation helpers (nblist.cu)
int gather_to_sorted3(Context* ctx, const float* a, const float* b, float* s6);
int scatter_from_sorted3(Context* ctx, const float* s6, float* a, float* b);
// the converged dipoles in caller order into the pinned h_stage ([2][n][3]),
// enqueued before a solve's synchronisation when stage_out is set
int stage_dipoles(Context* ctx);

}  // namespace t9gb

// the opaque handle of the C ABI
struct t9gb_context {
   t9gb::Context c;
};
