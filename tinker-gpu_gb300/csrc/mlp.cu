// Per-atom MLP for the learned initial guess of the induced dipoles:
// 32 inputs -> 64 SiLU -> 64 SiLU -> 3 outputs, BF16 weights and activations,
// FP32 accumulation, trained online with AdamW.
//
// Every contraction runs on the tensor cores through one hand-written GEMM
// (mma.sync m16n8k16 BF16 -> FP32): the forward layers, the backward input
// gradients and the weight gradients (split over the batch, partials summed
// in a fixed order, so training is bit-reproducible).  The reference has no
// learned component; the closest prior art is its AMOEBA+NN CELU network
// evaluated through cuBLAS Sgemm (src/nn.cpp:419-432).
#include <cuda_bf16.h>

#include <cmath>
#include <random>

#include "common.cuh"

namespace t9gb {

// ---------------------------------------------------------------------------
// GEMM: C[z][M][N] = sum over the z-th K chunk of A(m,k) B(k,n)
//   A(m,k) = TA ? A[k*lda + m] : A[m*lda + k]
//   B(k,n) = TB ? B[n*ldb + k] : B[k*ldb + n]
// Block tile 64 x 64 x 32, four warps of 16 rows x 64 columns.

__device__ __forceinline__ void mma_bf16_16816(float* d, const unsigned* a, const unsigned* b)
{
   asm volatile("mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
                "{%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

template <bool TA, bool TB>
__global__ void __launch_bounds__(128) k_gemm_bf16(int M, int N, int K, int kchunk, const __nv_bfloat16* __restrict__ A,
   int lda, const __nv_bfloat16* __restrict__ B, int ldb, float* __restrict__ C)
{
   __shared__ __align__(16) __nv_bfloat16 As[64][40];  // [m][k], rows padded to 80 B (conflict-free)
   __shared__ __align__(16) __nv_bfloat16 Bs[64][40];  // [n][k]
   const int tid = threadIdx.x, w = tid >> 5, lane = tid & 31, gq = lane >> 2, t4 = lane & 3;
   const int m0 = blockIdx.x * 64, n0 = blockIdx.y * 64;
   const int kbeg = blockIdx.z * kchunk, kend = min(K, kbeg + kchunk);
   float acc[8][4];
#pragma unroll
   for (int j = 0; j < 8; ++j)
      acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
   const __nv_bfloat16 zero = __float2bfloat16(0.f);
   for (int k0 = kbeg; k0 < kend; k0 += 32) {
      for (int e = tid; e < 64 * 32; e += 128) {
         int r, c;
         if (TA) {
            r = e % 64;
            c = e / 64;
         } else {
            r = e / 32;
            c = e % 32;
         }
         const int gm = m0 + r, gk = k0 + c;
         As[r][c] = (gm < M && gk < kend) ? (TA ? A[(size_t)gk * lda + gm] : A[(size_t)gm * lda + gk]) : zero;
      }
      for (int e = tid; e < 64 * 32; e += 128) {
         int r, c;
         if (TB) {
            r = e / 32;
            c = e % 32;
         } else {
            r = e % 64;
            c = e / 64;
         }
         const int gn = n0 + r, gk = k0 + c;
         Bs[r][c] = (gn < N && gk < kend) ? (TB ? B[(size_t)gn * ldb + gk] : B[(size_t)gk * ldb + gn]) : zero;
      }
      __syncthreads();
#pragma unroll
      for (int kk = 0; kk < 32; kk += 16) {
         unsigned a[4];
         const int r = 16 * w + gq;
         a[0] = *reinterpret_cast<const unsigned*>(&As[r][kk + 2 * t4]);
         a[1] = *reinterpret_cast<const unsigned*>(&As[r + 8][kk + 2 * t4]);
         a[2] = *reinterpret_cast<const unsigned*>(&As[r][kk + 8 + 2 * t4]);
         a[3] = *reinterpret_cast<const unsigned*>(&As[r + 8][kk + 8 + 2 * t4]);
#pragma unroll
         for (int j = 0; j < 8; ++j) {
            unsigned b[2];
            b[0] = *reinterpret_cast<const unsigned*>(&Bs[8 * j + gq][kk + 2 * t4]);
            b[1] = *reinterpret_cast<const unsigned*>(&Bs[8 * j + gq][kk + 8 + 2 * t4]);
            mma_bf16_16816(acc[j], a, b);
         }
      }
      __syncthreads();
   }
   float* Cz = C + (size_t)blockIdx.z * M * N;
   const int r0 = m0 + 16 * w + gq;
#pragma unroll
   for (int j = 0; j < 8; ++j) {
      const int c = n0 + 8 * j + 2 * t4;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
         const int r = r0 + 8 * h;
         if (r < M) {
            if (c < N)
               Cz[(size_t)r * N + c] = acc[j][2 * h];
            if (c + 1 < N)
               Cz[(size_t)r * N + c + 1] = acc[j][2 * h + 1];
         }
      }
   }
}

// out[i] = sum_z part[z][i] (fixed order)
__global__ void k_sum_splits(int size, int nsplit, const float* __restrict__ part, float* __restrict__ out)
{
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < size; i += gridDim.x * blockDim.x) {
      float v = 0.f;
#pragma unroll 8
      for (int z = 0; z < nsplit; ++z)
         v += part[(size_t)z * size + i];
      out[i] = v;
   }
}

static int gemm(Context* ctx, bool ta, bool tb, int M, int N, int K, const __nv_bfloat16* A, int lda,
   const __nv_bfloat16* B, int ldb, float* C, int nsplit)
{
   const int kchunk = ((K + nsplit - 1) / nsplit + 31) / 32 * 32;
   nsplit = (K + kchunk - 1) / kchunk;
   dim3 grid(grid_for(M, 64), grid_for(N, 64), nsplit);
   float* out = nsplit > 1 ? ctx->mlp.split : C;
   if (ta && !tb)
      k_gemm_bf16<true, false><<<grid, 128, 0, ctx->stream>>>(M, N, K, kchunk, A, lda, B, ldb, out);
   else if (!ta && tb)
      k_gemm_bf16<false, true><<<grid, 128, 0, ctx->stream>>>(M, N, K, kchunk, A, lda, B, ldb, out);
   else if (!ta && !tb)
      k_gemm_bf16<false, false><<<grid, 128, 0, ctx->stream>>>(M, N, K, kchunk, A, lda, B, ldb, out);
   else
      k_gemm_bf16<true, true><<<grid, 128, 0, ctx->stream>>>(M, N, K, kchunk, A, lda, B, ldb, out);
   if (nsplit > 1)
      k_sum_splits<<<grid_for(M * N, 256), 256, 0, ctx->stream>>>(M * N, nsplit, ctx->mlp.split, C);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// ---------------------------------------------------------------------------
// elementwise pieces

__device__ __forceinline__ float silu(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float silu_grad(float z)
{
   const float s = 1.f / (1.f + __expf(-z));
   return s * (1.f + z * (1.f - s));
}

// Z = C + b; H = silu(Z) (act) or Z, stored as BF16 (ldh columns, zero padded)
__global__ void k_bias_act(int rows, int N, int ldh, const float* __restrict__ C, const float* __restrict__ b,
   float* __restrict__ Z, __nv_bfloat16* __restrict__ H, int act)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < rows * ldh; e += gridDim.x * blockDim.x) {
      const int r = e / ldh, c = e % ldh;
      float z = 0.f;
      if (c < N)
         z = C[(size_t)r * N + c] + b[c];
      if (Z)
         Z[e] = z;
      if (H)
         H[e] = __float2bfloat16(act && c < N ? silu(z) : z);
   }
}

// dZ = dH * silu'(Z), BF16 out; f32 copy for the bias gradient
__global__ void k_silu_back(int size, const float* __restrict__ dH, const float* __restrict__ Z,
   __nv_bfloat16* __restrict__ dZ, float* __restrict__ dZf)
{
   for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < size; e += gridDim.x * blockDim.x) {
      const float v = dH[e] * silu_grad(Z[e]);
      dZ[e] = __float2bfloat16(v);
      dZf[e] = v;
   }
}

// MSE over the 3 outputs: dY = 2 (Y - T) / (rows * 3), zero in the padding
// columns and in rows whose rowpol[r % npad] is 0 (padding slots); per-row
// squared error for the loss
__global__ void k_loss_grad(int rows, const float* __restrict__ Y, const float* __restrict__ T,
   const float* __restrict__ rowpol, int npad, __nv_bfloat16* __restrict__ dY, float* __restrict__ dYf,
   double* __restrict__ err)
{
   for (int r = blockIdx.x * blockDim.x + threadIdx.x; r < rows; r += gridDim.x * blockDim.x) {
      double s = 0;
      const bool live = !rowpol || rowpol[r % npad] != 0.f;
      for (int c = 0; c < MLP_OUT_PAD; ++c) {
         float g = 0.f;
         if (c < MLP_OUT && live) {
            const float d = Y[(size_t)r * MLP_OUT_PAD + c] - T[(size_t)r * MLP_OUT + c];
            s += (double)d * d;
            g = 2.f * d / (float)(rows * MLP_OUT);
         }
         dY[(size_t)r * MLP_OUT_PAD + c] = __float2bfloat16(g);
         dYf[(size_t)r * MLP_OUT_PAD + c] = g;
      }
      err[r] = s;
   }
}

// Column sums of a [rows][N] f32 matrix (N <= 64), two fixed-order levels:
// COLSUM_BLOCKS blocks of 4 x 64 threads (column c = thread % 64, row group
// thread / 64) stride over the rows, then one block per column combines the
// block partials with a shared-memory tree.
constexpr int COLSUM_BLOCKS = 64;

__global__ void __launch_bounds__(256) k_colsum_part(int rows, int N, const float* __restrict__ X,
   float* __restrict__ part)
{
   __shared__ float sh[4][64];
   const int c = threadIdx.x & 63, g = threadIdx.x >> 6;
   float v = 0.f;
   if (c < N)
      for (int r = blockIdx.x * 4 + g; r < rows; r += COLSUM_BLOCKS * 4)
         v += X[(size_t)r * N + c];
   sh[g][c] = v;
   __syncthreads();
   if (g == 0 && c < N)
      part[(size_t)blockIdx.x * N + c] = (sh[0][c] + sh[1][c]) + (sh[2][c] + sh[3][c]);
}

__global__ void __launch_bounds__(COLSUM_BLOCKS) k_colsum_final(int N, const float* __restrict__ part,
   float* __restrict__ out)
{
   __shared__ float sh[COLSUM_BLOCKS];
   const int c = blockIdx.x;
   sh[threadIdx.x] = part[(size_t)threadIdx.x * N + c];
   __syncthreads();
   for (int o = COLSUM_BLOCKS / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o)
         sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
   }
   if (threadIdx.x == 0)
      out[c] = sh[0];
}

// fixed-order sum of a double array: block partials, then one block
__global__ void __launch_bounds__(256) k_sum_double_part(int n, const double* __restrict__ a,
   double* __restrict__ part)
{
   __shared__ double sh[256];
   double v = 0;
   for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
      v += a[i];
   sh[threadIdx.x] = v;
   __syncthreads();
   for (int o = blockDim.x / 2; o > 0; o >>= 1) {
      if (threadIdx.x < o)
         sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
   }
   if (threadIdx.x == 0)
      part[blockIdx.x] = sh[0];
}

__global__ void __launch_bounds__(64) k_sum_double_final(int nb, const double* __restrict__ part,
   double* __restrict__ out)
{
   __shared__ double sh[64];
   sh[threadIdx.x] = threadIdx.x < nb ? part[threadIdx.x] : 0.0;
   __syncthreads();
   for (int o = 32; o > 0; o >>= 1) {
      if (threadIdx.x < o)
         sh[threadIdx.x] += sh[threadIdx.x + o];
      __syncthreads();
   }
   if (threadIdx.x == 0)
      *out = sh[0];
}

// AdamW (Loshchilov & Hutter, 2019) on the FP32 master weights; refreshes
// the BF16 copies used by the GEMMs.  mask: parameters that stay zero (the
// padding columns of the output layer).  One block: the step count lives on
// the device (*step, incremented here) so a captured graph replays correctly.
__global__ void __launch_bounds__(1024) k_adamw(int size, float lr, float beta1, float beta2, float eps, float wd,
   int* __restrict__ step, float* __restrict__ w, const float* __restrict__ g, float* __restrict__ m,
   float* __restrict__ v, const unsigned char* __restrict__ mask, __nv_bfloat16* __restrict__ wb,
   const int* __restrict__ wb_index)
{
   const int t = *step + 1;
   const float c1 = 1.f - powf(beta1, (float)t), c2 = 1.f - powf(beta2, (float)t);
   for (int i = threadIdx.x; i < size; i += blockDim.x) {
      if (!mask[i])
         continue;
      const float gi = g[i];
      const float mi = beta1 * m[i] + (1.f - beta1) * gi;
      const float vi = beta2 * v[i] + (1.f - beta2) * gi * gi;
      m[i] = mi;
      v[i] = vi;
      float wi = w[i];
      wi -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * wi);
      w[i] = wi;
      if (wb_index[i] >= 0)
         wb[wb_index[i]] = __float2bfloat16(wi);
   }
   __syncthreads();
   if (threadIdx.x == 0)
      *step = t;
}

// ---------------------------------------------------------------------------
// parameter layout (FP32 master vector):
//   W1 [32][64] | b1 [64] | W2 [64][64] | b2 [64] | W3 [64][8] | b3 [8]
// BF16 copies: W1 | W2 | W3 in the same order (weights only).

constexpr int OFF_W1 = 0;
constexpr int OFF_B1 = OFF_W1 + MLP_IN * MLP_HID;
constexpr int OFF_W2 = OFF_B1 + MLP_HID;
constexpr int OFF_B2 = OFF_W2 + MLP_HID * MLP_HID;
constexpr int OFF_W3 = OFF_B2 + MLP_HID;
constexpr int OFF_B3 = OFF_W3 + MLP_HID * MLP_OUT_PAD;
constexpr int OFF_END = OFF_B3 + MLP_OUT_PAD;
constexpr int BF_W1 = 0, BF_W2 = BF_W1 + MLP_IN * MLP_HID, BF_W3 = BF_W2 + MLP_HID * MLP_HID;
constexpr int BF_END = BF_W3 + MLP_HID * MLP_OUT_PAD;
static_assert(OFF_END == MLP_NPARAM, "parameter count");

int mlp_init(Context* ctx, unsigned seed);

// allocate for max_rows rows (kept when large enough) and initialise
int mlp_alloc(Context* ctx, int max_rows, unsigned seed)
{
   MlpState& S = ctx->mlp;
   if (S.w && S.max_rows >= max_rows)
      return mlp_init(ctx, seed);
   mlp_free(ctx);
   S.max_rows = max_rows;
   T9_CUDA(cudaMalloc(&S.step, sizeof(int)));
   T9_CUDA(cudaMalloc(&S.w, sizeof(float) * MLP_NPARAM));
   T9_CUDA(cudaMalloc(&S.g, sizeof(float) * MLP_NPARAM));
   T9_CUDA(cudaMalloc(&S.m, sizeof(float) * MLP_NPARAM));
   T9_CUDA(cudaMalloc(&S.v, sizeof(float) * MLP_NPARAM));
   T9_CUDA(cudaMalloc(&S.mask, MLP_NPARAM));
   T9_CUDA(cudaMalloc(&S.wb_index, sizeof(int) * MLP_NPARAM));
   T9_CUDA(cudaMalloc(&S.wb, sizeof(__nv_bfloat16) * BF_END));
   const size_t R = max_rows;
   T9_CUDA(cudaMalloc(&S.x, sizeof(__nv_bfloat16) * R * MLP_IN));
   T9_CUDA(cudaMalloc(&S.z1, sizeof(float) * R * MLP_HID));
   T9_CUDA(cudaMalloc(&S.z2, sizeof(float) * R * MLP_HID));
   T9_CUDA(cudaMalloc(&S.h1, sizeof(__nv_bfloat16) * R * MLP_HID));
   T9_CUDA(cudaMalloc(&S.h2, sizeof(__nv_bfloat16) * R * MLP_HID));
   T9_CUDA(cudaMalloc(&S.c, sizeof(float) * R * MLP_HID));
   T9_CUDA(cudaMalloc(&S.y, sizeof(float) * R * MLP_OUT_PAD));
   T9_CUDA(cudaMalloc(&S.t, sizeof(float) * R * MLP_OUT));
   T9_CUDA(cudaMalloc(&S.dy, sizeof(__nv_bfloat16) * R * MLP_OUT_PAD));
   T9_CUDA(cudaMalloc(&S.dyf, sizeof(float) * R * MLP_OUT_PAD));
   T9_CUDA(cudaMalloc(&S.dz, sizeof(__nv_bfloat16) * R * MLP_HID));
   T9_CUDA(cudaMalloc(&S.dzf, sizeof(float) * R * MLP_HID));
   T9_CUDA(cudaMalloc(&S.err, sizeof(double) * R));
   T9_CUDA(cudaMalloc(&S.loss, sizeof(double)));
   S.nsplit = 128;
   T9_CUDA(cudaMalloc(&S.split, sizeof(float) * (size_t)std::max<size_t>(S.nsplit * MLP_HID * MLP_HID, 1024 * MLP_HID)));
   T9_CUDA(cudaMalloc(&S.gpart, sizeof(float) * ((R + 127) / 128) * MLP_NPARAM));  // 128-row tiles
   return mlp_init(ctx, seed);
}

// seeded Glorot-uniform weights, zero biases, optimiser state cleared
int mlp_init(Context* ctx, unsigned seed)
{
   MlpState& S = ctx->mlp;
   std::vector<float> w(MLP_NPARAM, 0.f);
   std::vector<unsigned char> mask(MLP_NPARAM, 1);
   std::vector<int> idx(MLP_NPARAM, -1);
   std::mt19937 rng(seed);
   auto fill = [&](int off, int bf, int fin, int fout, int cols_used) {
      const float lim = std::sqrt(6.f / (fin + cols_used));
      std::uniform_real_distribution<float> U(-lim, lim);
      for (int r = 0; r < fin; ++r)
         for (int c = 0; c < fout; ++c) {
            const int i = off + r * fout + c;
            idx[i] = bf + r * fout + c;
            if (c < cols_used)
               w[i] = U(rng);
            else
               mask[i] = 0;
         }
   };
   fill(OFF_W1, BF_W1, MLP_IN, MLP_HID, MLP_HID);
   fill(OFF_W2, BF_W2, MLP_HID, MLP_HID, MLP_HID);
   fill(OFF_W3, BF_W3, MLP_HID, MLP_OUT_PAD, MLP_OUT);
   for (int c = MLP_OUT; c < MLP_OUT_PAD; ++c)
      mask[OFF_B3 + c] = 0;
   T9_CUDA(cudaMemcpyAsync(S.mask, mask.data(), MLP_NPARAM, cudaMemcpyHostToDevice, ctx->stream));
   T9_CUDA(cudaMemcpyAsync(S.wb_index, idx.data(), sizeof(int) * MLP_NPARAM, cudaMemcpyHostToDevice, ctx->stream));
   T9_CHECK(mlp_set_weights(ctx, w.data()));
   return T9GB_OK;
}

void mlp_free(Context* ctx)
{
   MlpState& S = ctx->mlp;
   void* p[] = {S.step, S.w, S.g, S.m, S.v, S.mask, S.wb_index, S.wb, S.x, S.z1, S.z2, S.h1, S.h2, S.c, S.y, S.t, S.dy,
      S.dyf, S.dz, S.dzf, S.err, S.loss, S.split, S.gpart};
   for (void* q : p)
      if (q)
         cudaFree(q);
   S = MlpState();
}

// master weights from the host; resets the optimiser moments
int mlp_set_weights(Context* ctx, const float* w_host)
{
   MlpState& S = ctx->mlp;
   std::vector<float> w(w_host, w_host + MLP_NPARAM);
   std::vector<__nv_bfloat16> wb(BF_END);
   auto cp = [&](int off, int bf, int size) {
      for (int i = 0; i < size; ++i)
         wb[bf + i] = __float2bfloat16(w[off + i]);
   };
   cp(OFF_W1, BF_W1, MLP_IN * MLP_HID);
   cp(OFF_W2, BF_W2, MLP_HID * MLP_HID);
   cp(OFF_W3, BF_W3, MLP_HID * MLP_OUT_PAD);
   cudaStream_t st = ctx->stream;
   T9_CUDA(cudaMemcpyAsync(S.w, w.data(), sizeof(float) * MLP_NPARAM, cudaMemcpyHostToDevice, st));
   T9_CUDA(cudaMemcpyAsync(S.wb, wb.data(), sizeof(__nv_bfloat16) * BF_END, cudaMemcpyHostToDevice, st));
   T9_CUDA(cudaMemsetAsync(S.m, 0, sizeof(float) * MLP_NPARAM, st));
   T9_CUDA(cudaMemsetAsync(S.v, 0, sizeof(float) * MLP_NPARAM, st));
   T9_CUDA(cudaMemsetAsync(S.step, 0, sizeof(int), st));
   T9_CUDA(cudaStreamSynchronize(st));  // the host vectors go out of scope
   return T9GB_OK;
}

int mlp_get_weights(Context* ctx, float* w_host)
{
   T9_CUDA(cudaMemcpyAsync(w_host, ctx->mlp.w, sizeof(float) * MLP_NPARAM, cudaMemcpyDeviceToHost, ctx->stream));
   T9_CUDA(cudaStreamSynchronize(ctx->stream));
   return T9GB_OK;
}

// ---------------------------------------------------------------------------
// Forward pass on the fifth-generation tensor cores (tcgen05): one CTA of
// four warps per 128 rows.  The row tile and the transposed weights are
// staged in shared memory in the canonical K-major layout without swizzle
// (8-row x 16-byte core matrices; LBO = 128 B between core matrices along K,
// SBO = K / 8 x 128 B between 8-row groups), one thread issues the
// tcgen05.mma instructions (M = 128, K = 16 per instruction, BF16 in, FP32
// accumulated in tensor memory), tcgen05.commit signals an mbarrier, and each
// warp reads its 32 rows back with tcgen05.ld for the bias + SiLU epilogue,
// which writes the next layer's operand tile.  The outputs are those of the
// mma.sync path (z1, h1, z2, h2, y), equal to them up to the order of the
// FP32 accumulation inside the MMA.

constexpr int TC_ROWS = 128;  // also the tile of S.gpart
constexpr int TC_TMEM_COLS = 128;  // D1 in columns 0-63, D2 in 64-127, D3 in 0-15

// byte offset of element (r, k) in a K-major no-swizzle tile with K columns
__device__ __forceinline__ int kmaj_off(int r, int k, int K)
{
   return ((r >> 3) * (K >> 3) + (k >> 3)) * 128 + (r & 7) * 16 + (k & 7) * 2;
}

// shared-memory matrix descriptor: start address, LBO, SBO (all >> 4), the
// fixed 0b001 at bits 46-48, no swizzle
__device__ __forceinline__ unsigned long long smem_desc(unsigned addr, int K)
{
   const unsigned long long lbo = 128 >> 4, sbo = (unsigned long long)((K >> 3) * 128) >> 4;
   return (unsigned long long)((addr & 0x3ffff) >> 4) | (lbo << 16) | (sbo << 32) | (1ull << 46);
}

// kind::f16 instruction descriptor: D f32, A and B bf16, both K-major, N, M = 128
__host__ __device__ constexpr unsigned tc_idesc(int n)
{
   return (1u << 4) | (1u << 7) | (1u << 10) | ((unsigned)(n >> 3) << 17) | ((unsigned)(TC_ROWS >> 4) << 24);
}

__device__ __forceinline__ void tc_mma(unsigned dtmem, unsigned long long adesc, unsigned long long bdesc,
   unsigned idesc, int accum)
{
   asm volatile("{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
                " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(dtmem),
                "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accum)
                : "memory");
}

__device__ __forceinline__ void tc_commit(unsigned bar)
{
   asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar)
                : "memory");
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes
__device__ __forceinline__ void tc_ld16(unsigned taddr, float* v)
{
   unsigned r[16];
   asm volatile("tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, "
                "%13, %14, %15}, [%16];\n"
                : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
                "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
                : "r"(taddr));
   asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
   for (int i = 0; i < 16; ++i)
      v[i] = __uint_as_float(r[i]);
}

// operand tiles (bytes): X [128][32], H1 / H2 [128][64], W1^T [64][32],
// W2^T [64][64], W3^T [16][64] (columns 8-15 zero)
constexpr int TC_SX = 0, TC_SH1 = TC_SX + 128 * 32 * 2, TC_SH2 = TC_SH1 + 128 * 64 * 2;
constexpr int TC_SW1 = TC_SH2 + 128 * 64 * 2, TC_SW2 = TC_SW1 + 64 * 32 * 2, TC_SW3 = TC_SW2 + 64 * 64 * 2;
constexpr int TC_SMEM = TC_SW3 + 16 * 64 * 2;  // 55,296 bytes: at most four CTAs per SM, 4 x 128 TMEM columns
// with the activations kept: a [128][65] FP32 staging tile for coalesced
// stores of z (88,576 bytes: at most two CTAs per SM)
constexpr int TC_ZLD = MLP_HID + 1;
constexpr int TC_SMEM_ACT = TC_SMEM + TC_ROWS * TC_ZLD * 4;

// ACT: also store z1, h1, z2, h2 (the backward pass reads them); the
// inference forward stores only y
template <bool ACT>
__global__ void __launch_bounds__(128) k_mlp_forward_tc(int rows, const __nv_bfloat16* __restrict__ x,
   const __nv_bfloat16* __restrict__ wb, const float* __restrict__ w, float* __restrict__ z1,
   __nv_bfloat16* __restrict__ h1, float* __restrict__ z2, __nv_bfloat16* __restrict__ h2, float* __restrict__ y,
   int* __restrict__ err)
{
   extern __shared__ __align__(128) unsigned char tsm[];
   __shared__ __align__(8) unsigned long long bar;
   __shared__ unsigned tmem_slot;
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int r0 = blockIdx.x * TC_ROWS;
   const unsigned base = (unsigned)__cvta_generic_to_shared(tsm);
   const unsigned bar_s = (unsigned)__cvta_generic_to_shared(&bar);

   // tensor memory for the accumulators (warp 0 allocates, and frees at the end)
   if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                      (unsigned)__cvta_generic_to_shared(&tmem_slot)),
                   "r"((unsigned)TC_TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   if (tid == 0)
      mbar_init(bar_s, 1);
   // operand tiles: the input rows and the transposed weights
   for (int e = tid; e < TC_ROWS * MLP_IN; e += 128) {
      const int r = e / MLP_IN, k = e % MLP_IN;
      const __nv_bfloat16 v = r0 + r < rows ? x[(size_t)(r0 + r) * MLP_IN + k] : __float2bfloat16(0.f);
      *reinterpret_cast<__nv_bfloat16*>(tsm + TC_SX + kmaj_off(r, k, MLP_IN)) = v;
   }
   // the weights are read in memory order (W[k][n], n fastest: coalesced)
   // and stored transposed, (n, k) = W[k][n]
   for (int e = tid; e < MLP_IN * MLP_HID; e += 128) {
      const int k = e / MLP_HID, n = e % MLP_HID;
      *reinterpret_cast<__nv_bfloat16*>(tsm + TC_SW1 + kmaj_off(n, k, MLP_IN)) = wb[BF_W1 + e];
   }
   for (int e = tid; e < MLP_HID * MLP_HID; e += 128) {
      const int k = e / MLP_HID, n = e % MLP_HID;
      *reinterpret_cast<__nv_bfloat16*>(tsm + TC_SW2 + kmaj_off(n, k, MLP_HID)) = wb[BF_W2 + e];
   }
   for (int e = tid; e < MLP_HID * 16; e += 128) {
      const int k = e / 16, n = e % 16;
      *reinterpret_cast<__nv_bfloat16*>(tsm + TC_SW3 + kmaj_off(n, k, MLP_HID)) =
         n < MLP_OUT_PAD ? wb[BF_W3 + k * MLP_OUT_PAD + n] : __float2bfloat16(0.f);
   }
   // the tiles (generic proxy) before the tensor core reads them (async proxy)
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const unsigned tmem = tmem_slot;
   const unsigned lane_base = tmem + ((unsigned)(32 * warp) << 16);
   const int r = r0 + 32 * warp + lane;  // this thread's row
   unsigned phase = 0;

   // one layer: D[columns dcol..] = A B over K (K / 16 MMAs), then wait
   auto layer = [&](unsigned a_off, unsigned b_off, int K, int n, unsigned dcol) {
      if (tid == 0) {
         for (int kk = 0; kk < K / 16; ++kk)
            tc_mma(tmem + dcol, smem_desc(base + a_off + kk * 256, K), smem_desc(base + b_off + kk * 256, K),
               tc_idesc(n), kk > 0);
         tc_commit(bar_s);
      }
      if (!mbar_wait_bounded(bar_s, phase)) {
         // record it, and give the MMAs in flight a second bounded wait
         // before their operands and accumulators are reused or freed
         if (tid == 0)
            atomicOr(err, 4);
         mbar_wait_bounded(bar_s, phase);
      }
      phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   };

   // hidden layer epilogue: z = D + b, h = silu(z) into the next operand
   // tile; ACT: z through the staging tile, then z and h stored row-major
   // with consecutive threads on consecutive columns
   float* zst = reinterpret_cast<float*>(tsm + TC_SMEM);
   auto hidden = [&](unsigned dcol, const float* b, float* zg, __nv_bfloat16* hg, unsigned h_off) {
#pragma unroll
      for (int c0 = 0; c0 < MLP_HID; c0 += 16) {
         float v[16];
         tc_ld16(lane_base + dcol + c0, v);
#pragma unroll
         for (int i = 0; i < 16; ++i) {
            const int c = c0 + i;
            const float z = v[i] + b[c];
            const __nv_bfloat16 hv = __float2bfloat16(silu(z));
            if (ACT)
               zst[(32 * warp + lane) * TC_ZLD + c] = z;
            *reinterpret_cast<__nv_bfloat16*>(tsm + h_off + kmaj_off(32 * warp + lane, c, MLP_HID)) =
               r < rows ? hv : __float2bfloat16(0.f);
         }
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      if (ACT) {
         for (int e = tid; e < TC_ROWS * MLP_HID; e += 128) {
            const int rl = e / MLP_HID, c = e % MLP_HID;
            if (r0 + rl < rows) {
               zg[(size_t)(r0 + rl) * MLP_HID + c] = zst[rl * TC_ZLD + c];
               hg[(size_t)(r0 + rl) * MLP_HID + c] =
                  *reinterpret_cast<const __nv_bfloat16*>(tsm + h_off + kmaj_off(rl, c, MLP_HID));
            }
         }
         __syncthreads();  // the staging tile is reused by the next layer
      }
   };

   layer(TC_SX, TC_SW1, MLP_IN, MLP_HID, 0);
   hidden(0, w + OFF_B1, z1, h1, TC_SH1);
   layer(TC_SH1, TC_SW2, MLP_HID, MLP_HID, 64);
   hidden(64, w + OFF_B2, z2, h2, TC_SH2);
   layer(TC_SH2, TC_SW3, MLP_HID, 16, 0);
   {
      float v[16];
      tc_ld16(lane_base, v);
      if (r < rows)
#pragma unroll
         for (int c = 0; c < MLP_OUT_PAD; ++c)
            y[(size_t)r * MLP_OUT_PAD + c] = v[c] + w[OFF_B3 + c];
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   if (warp == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((unsigned)TC_TMEM_COLS)
                   : "memory");
   }
}

// ---------------------------------------------------------------------------
// Backward pass on tcgen05: one CTA of four warps per 128 rows computes the
// loss gradient dY, the hidden deltas dZ2 = (dY W3^T) silu'(z2) and
// dZ1 = (dZ2 W2^T) silu'(z1), and this tile's weight gradients
// dW3 = H2^T dY, dW2 = H1^T dZ2, dW1 = X^T dZ1 (the transposed activations
// padded to 128 rows, so every MMA has M = 128), plus the bias-gradient
// column sums and the squared error; it writes them as one partial vector
// per CTA, which k_grad_reduce adds in a fixed order.  The BF16 rounding
// points are those of the mma.sync path (dY and the deltas rounded for the
// products, kept in FP32 for the bias sums).
constexpr int TB_SXT = 0;                              // X^T pad   [128][128]
constexpr int TB_SH1T = TB_SXT + 128 * 128 * 2;        // H1^T pad  [128][128]
constexpr int TB_SH2T = TB_SH1T + 128 * 128 * 2;       // H2^T pad  [128][128]
constexpr int TB_SW3 = TB_SH2T + 128 * 128 * 2;        // W3 as B   [64][16]
constexpr int TB_SW2 = TB_SW3 + 64 * 16 * 2;           // W2 as B   [64][64]
constexpr int TB_SDY = TB_SW2 + 64 * 64 * 2;           // dY        [128][16]
constexpr int TB_SDYT = TB_SDY + 128 * 16 * 2;         // dY^T      [16][128]
constexpr int TB_SDZ = TB_SDYT + 16 * 128 * 2;         // dZ2       [128][64]
constexpr int TB_SDZT = TB_SDZ + 128 * 64 * 2;         // dZ^T      [64][128]
constexpr int TB_SZ = TB_SDZT + 64 * 128 * 2;          // z staging [128][65] f32
constexpr int TB_SB = TB_SZ + 128 * TC_ZLD * 4;        // bias partials [4 warps][8 + 64 + 64] f32
constexpr int TB_SMEM = TB_SB + 4 * (8 + 64 + 64) * 4; // 184,960 bytes: one CTA per SM
static_assert(TB_SMEM == 184960, "backward tile layout");
constexpr int TB_TMEM_COLS = 512;  // dH2 0-63, dW3 64-79, dH1 128-191, dW2 192-255, dW1 256-319

// column sums of one value per lane and column over a warp (butterfly: every
// lane ends with the sum; lane 0 stores it)
template <int N>
__device__ __forceinline__ void warp_colsum(const float* v, float* out, int lane)
{
#pragma unroll
   for (int c = 0; c < N; ++c) {
      float a = v[c];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0)
         out[c] = a;
   }
}

__global__ void __launch_bounds__(128) k_mlp_backward_tc(int rows, int npad, const float* __restrict__ rowpol,
   const __nv_bfloat16* __restrict__ x, const float* __restrict__ z1, const __nv_bfloat16* __restrict__ h1,
   const float* __restrict__ z2, const __nv_bfloat16* __restrict__ h2, const float* __restrict__ y,
   const float* __restrict__ t, const __nv_bfloat16* __restrict__ wb, float* __restrict__ gpart,
   double* __restrict__ lpart, int* __restrict__ err)
{
   extern __shared__ __align__(128) unsigned char bsm[];
   __shared__ __align__(8) unsigned long long bar;
   __shared__ unsigned tmem_slot;
   __shared__ double lsum[4];
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int r0 = blockIdx.x * TC_ROWS;
   const int rl = 32 * warp + lane, r = r0 + rl;  // this thread's row
   const unsigned base = (unsigned)__cvta_generic_to_shared(bsm);
   const unsigned bar_s = (unsigned)__cvta_generic_to_shared(&bar);
   float* zst = reinterpret_cast<float*>(bsm + TB_SZ);
   float* bpart = reinterpret_cast<float*>(bsm + TB_SB);
   auto bf = [&](int off, int rr, int k, int K) -> __nv_bfloat16& {
      return *reinterpret_cast<__nv_bfloat16*>(bsm + off + kmaj_off(rr, k, K));
   };

   if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                      (unsigned)__cvta_generic_to_shared(&tmem_slot)),
                   "r"((unsigned)TB_TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   if (tid == 0)
      mbar_init(bar_s, 1);
   const __nv_bfloat16 zero = __float2bfloat16(0.f);
   // transposed activation tiles, rows past the data zero
   for (int e = tid; e < 128 * 128; e += 128) {
      const int m = e / 128, k = e % 128;
      if (m >= MLP_IN)
         bf(TB_SXT, m, k, 128) = zero;
      if (m >= MLP_HID) {
         bf(TB_SH1T, m, k, 128) = zero;
         bf(TB_SH2T, m, k, 128) = zero;
      }
   }
   for (int e = tid; e < TC_ROWS * MLP_IN; e += 128) {  // (m = i, k = row) = x[row][i]
      const int rr = e / MLP_IN, i = e % MLP_IN;
      bf(TB_SXT, i, rr, 128) = r0 + rr < rows ? x[(size_t)(r0 + rr) * MLP_IN + i] : zero;
   }
   for (int e = tid; e < TC_ROWS * MLP_HID; e += 128) {
      const int rr = e / MLP_HID, h = e % MLP_HID;
      const bool in = r0 + rr < rows;
      bf(TB_SH1T, h, rr, 128) = in ? h1[(size_t)(r0 + rr) * MLP_HID + h] : zero;
      bf(TB_SH2T, h, rr, 128) = in ? h2[(size_t)(r0 + rr) * MLP_HID + h] : zero;
      zst[rr * TC_ZLD + h] = in ? z2[(size_t)(r0 + rr) * MLP_HID + h] : 0.f;
   }
   for (int e = tid; e < MLP_HID * 16; e += 128) {  // (n = h, k = o) = W3[h][o]
      const int h = e / 16, o = e % 16;
      bf(TB_SW3, h, o, 16) = o < MLP_OUT_PAD ? wb[BF_W3 + h * MLP_OUT_PAD + o] : zero;
   }
   for (int e = tid; e < MLP_HID * MLP_HID; e += 128) {  // (n = h1, k = h2) = W2[h1][h2]
      const int a = e / MLP_HID, b = e % MLP_HID;
      bf(TB_SW2, a, b, MLP_HID) = wb[BF_W2 + e];
   }
   // loss gradient of this row (k_loss_grad): dY = 2 (y - t) / (3 rows)
   const bool live = r < rows && (!rowpol || rowpol[r % npad] != 0.f);
   double se = 0;
   float dyf[MLP_OUT_PAD];
#pragma unroll
   for (int c = 0; c < MLP_OUT_PAD; ++c) {
      float g = 0.f;
      if (c < MLP_OUT && live) {
         const float d = y[(size_t)r * MLP_OUT_PAD + c] - t[(size_t)r * MLP_OUT + c];
         se += (double)d * d;
         g = 2.f * d / (float)(rows * MLP_OUT);
      }
      dyf[c] = g;
   }
#pragma unroll
   for (int c = 0; c < 16; ++c) {
      const __nv_bfloat16 v = c < MLP_OUT_PAD ? __float2bfloat16(dyf[c]) : zero;
      bf(TB_SDY, rl, c, 16) = v;
      bf(TB_SDYT, c, rl, 128) = v;
   }
   // bias column sums over the tile: per warp here, across the four warps at the end
   warp_colsum<MLP_OUT_PAD>(dyf, bpart + warp * 136, lane);
   {
      double a = se;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0)
         lsum[warp] = a;
   }
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const unsigned tmem = tmem_slot;
   const unsigned lane_base = tmem + ((unsigned)(32 * warp) << 16);
   unsigned phase = 0;
   auto mmas = [&](unsigned dcol, unsigned a_off, int KA, unsigned b_off, int K, int n) {
      for (int kk = 0; kk < K / 16; ++kk)
         tc_mma(tmem + dcol, smem_desc(base + a_off + kk * 256, KA), smem_desc(base + b_off + kk * 256, KA),
            tc_idesc(n), kk > 0);
   };
   auto wait = [&]() {
      if (!mbar_wait_bounded(bar_s, phase)) {
         if (tid == 0)
            atomicOr(err, 4);
         mbar_wait_bounded(bar_s, phase);
      }
      phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   };
   auto sync_tiles = [&]() {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   };
   // dH2 = dY W3^T (K = 16), dW3 = H2^T dY (K = 128 rows)
   if (tid == 0) {
      mmas(0, TB_SDY, 16, TB_SW3, 16, MLP_HID);
      mmas(64, TB_SH2T, 128, TB_SDYT, 128, 16);
      tc_commit(bar_s);
   }
   wait();
   // hidden delta 2 (k_silu_back): dZ2 = dH2 silu'(z2); z2 from the staging tile
   float dz[16];
   auto delta = [&](unsigned dcol, int bias_off) {
      float cs[MLP_HID];
#pragma unroll
      for (int c0 = 0; c0 < MLP_HID; c0 += 16) {
         tc_ld16(lane_base + dcol + c0, dz);
#pragma unroll
         for (int i = 0; i < 16; ++i) {
            const int c = c0 + i;
            const float v = r < rows ? dz[i] * silu_grad(zst[rl * TC_ZLD + c]) : 0.f;
            cs[c] = v;
            const __nv_bfloat16 vb = __float2bfloat16(v);
            bf(TB_SDZ, rl, c, MLP_HID) = vb;
            bf(TB_SDZT, c, rl, 128) = vb;
         }
      }
      warp_colsum<MLP_HID>(cs, bpart + warp * 136 + bias_off, lane);
   };
   delta(0, 8);
   __syncthreads();  // every thread done with z2 before z1 replaces it
   for (int e = tid; e < TC_ROWS * MLP_HID; e += 128) {
      const int rr = e / MLP_HID, h = e % MLP_HID;
      zst[rr * TC_ZLD + h] = r0 + rr < rows ? z1[(size_t)(r0 + rr) * MLP_HID + h] : 0.f;
   }
   sync_tiles();
   // dH1 = dZ2 W2^T (K = 64), dW2 = H1^T dZ2 (K = 128 rows)
   if (tid == 0) {
      mmas(128, TB_SDZ, MLP_HID, TB_SW2, MLP_HID, MLP_HID);
      mmas(192, TB_SH1T, 128, TB_SDZT, 128, MLP_HID);
      tc_commit(bar_s);
   }
   wait();
   // hidden delta 1: dZ1 = dH1 silu'(z1) into the dZ^T tile (dW2 has read it)
   delta(128, 72);
   sync_tiles();
   // dW1 = X^T dZ1 (K = 128 rows)
   if (tid == 0) {
      mmas(256, TB_SXT, 128, TB_SDZT, 128, MLP_HID);
      tc_commit(bar_s);
   }
   wait();
   // this tile's gradient vector, in the parameter layout of S.g
   float* gp = gpart + (size_t)blockIdx.x * MLP_NPARAM;
   if (warp < 2) {  // TMEM lanes 0-63: dW3 rows h, dW2 rows h1
      float v[16];
      tc_ld16(lane_base + 64, v);
#pragma unroll
      for (int o = 0; o < MLP_OUT_PAD; ++o)
         gp[OFF_W3 + rl * MLP_OUT_PAD + o] = v[o];
#pragma unroll
      for (int c0 = 0; c0 < MLP_HID; c0 += 16) {
         tc_ld16(lane_base + 192 + c0, v);
#pragma unroll
         for (int i = 0; i < 16; ++i)
            gp[OFF_W2 + rl * MLP_HID + c0 + i] = v[i];
      }
   }
   if (warp == 0) {  // TMEM lanes 0-31: dW1 rows i
      float v[16];
#pragma unroll
      for (int c0 = 0; c0 < MLP_HID; c0 += 16) {
         tc_ld16(lane_base + 256 + c0, v);
#pragma unroll
         for (int i = 0; i < 16; ++i)
            gp[OFF_W1 + rl * MLP_HID + c0 + i] = v[i];
      }
   }
   __syncthreads();
   for (int c = tid; c < 136; c += 128) {
      const float a = (bpart[c] + bpart[136 + c]) + (bpart[272 + c] + bpart[408 + c]);
      if (c < 8)
         gp[OFF_B3 + c] = a;
      else if (c < 72)
         gp[OFF_B2 + c - 8] = a;
      else
         gp[OFF_B1 + c - 72] = a;
   }
   if (tid == 0)
      lpart[blockIdx.x] = (lsum[0] + lsum[1]) + (lsum[2] + lsum[3]);
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   if (warp == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((unsigned)TB_TMEM_COLS)
                   : "memory");
   }
}

int mlp_tc_setup()
{
   return cudaFuncSetAttribute(k_mlp_backward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TB_SMEM) ==
            cudaSuccess &&
         cudaFuncSetAttribute(k_mlp_forward_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM_ACT) ==
            cudaSuccess &&
         cudaFuncSetAttribute(k_mlp_forward_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM) ==
            cudaSuccess
      ? T9GB_OK
      : T9GB_CUDA_ERR;
}

// fixed-order sum of the per-CTA partial gradients (and, in one thread, of
// the squared errors); the padding parameters stay zero
__global__ void __launch_bounds__(256) k_grad_reduce(int ncta, const float* __restrict__ gpart,
   const double* __restrict__ lpart, const unsigned char* __restrict__ mask, float* __restrict__ g,
   double* __restrict__ loss)
{
   const int p = blockIdx.x * blockDim.x + threadIdx.x;
   if (p < MLP_NPARAM) {
      float a = 0.f;
      for (int c = 0; c < ncta; ++c)
         a += gpart[(size_t)c * MLP_NPARAM + p];
      g[p] = mask[p] ? a : 0.f;
   }
   if (p == 0) {
      double l = 0;
      for (int c = 0; c < ncta; ++c)
         l += lpart[c];
      *loss = l;
   }
}

// forward over rows of S.x; outputs in S.y [rows][8]; act: also the
// activations the backward pass reads (the tcgen05 path leaves them out
// otherwise; the mma.sync path always keeps them)
int mlp_forward(Context* ctx, int rows, bool act)
{
   MlpState& S = ctx->mlp;
   const __nv_bfloat16* wb = reinterpret_cast<const __nv_bfloat16*>(S.wb);
   if (ctx->mlp_tc) {
      auto k = act ? k_mlp_forward_tc<true> : k_mlp_forward_tc<false>;
      k<<<grid_for(rows, TC_ROWS), 128, act ? TC_SMEM_ACT : TC_SMEM, ctx->stream>>>(rows, S.x, wb, S.w, S.z1, S.h1,
         S.z2, S.h2, S.y, ctx->copy_err);
      T9_CUDA(cudaGetLastError());
      return T9GB_OK;
   }
   T9_CHECK(gemm(ctx, false, false, rows, MLP_HID, MLP_IN, S.x, MLP_IN, wb + BF_W1, MLP_HID, S.c, 1));
   k_bias_act<<<grid_for((long long)rows * MLP_HID, 256), 256, 0, ctx->stream>>>(rows, MLP_HID, MLP_HID, S.c,
      S.w + OFF_B1, S.z1, S.h1, 1);
   T9_CHECK(gemm(ctx, false, false, rows, MLP_HID, MLP_HID, S.h1, MLP_HID, wb + BF_W2, MLP_HID, S.c, 1));
   k_bias_act<<<grid_for((long long)rows * MLP_HID, 256), 256, 0, ctx->stream>>>(rows, MLP_HID, MLP_HID, S.c,
      S.w + OFF_B2, S.z2, S.h2, 1);
   T9_CHECK(gemm(ctx, false, false, rows, MLP_OUT_PAD, MLP_HID, S.h2, MLP_HID, wb + BF_W3, MLP_OUT_PAD, S.c, 1));
   k_bias_act<<<grid_for((long long)rows * MLP_OUT_PAD, 256), 256, 0, ctx->stream>>>(rows, MLP_OUT_PAD,
      MLP_OUT_PAD, S.c, S.w + OFF_B3, S.y, nullptr, 0);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// loss and full gradient for rows of S.x with targets S.t (after forward);
// gradient in S.g, summed squared error in S.loss.  rowpol (may be null):
// rows r with rowpol[r % npad] == 0 are left out.
int mlp_backward(Context* ctx, int rows, const float* rowpol, int npad)
{
   MlpState& S = ctx->mlp;
   const __nv_bfloat16* wb = reinterpret_cast<const __nv_bfloat16*>(S.wb);
   if (ctx->mlp_tc) {
      // one fused pass per 128 rows, then the fixed-order tile sum; the
      // per-tile squared errors go to the front of S.err
      const int ncta = (rows + TC_ROWS - 1) / TC_ROWS;
      k_mlp_backward_tc<<<ncta, 128, TB_SMEM, ctx->stream>>>(rows, npad, rowpol, S.x, S.z1, S.h1, S.z2, S.h2, S.y,
         S.t, wb, S.gpart, S.err, ctx->copy_err);
      k_grad_reduce<<<(MLP_NPARAM + 255) / 256, 256, 0, ctx->stream>>>(ncta, S.gpart, S.err, S.mask, S.g, S.loss);
      T9_CUDA(cudaGetLastError());
      return T9GB_OK;
   }
   const int ns = S.nsplit;
   k_loss_grad<<<grid_for(rows, 256), 256, 0, ctx->stream>>>(rows, S.y, S.t, rowpol, npad, S.dy, S.dyf,
      S.err);
   double* dpart = reinterpret_cast<double*>(S.split);
   k_sum_double_part<<<64, 256, 0, ctx->stream>>>(rows, S.err, dpart);
   k_sum_double_final<<<1, 64, 0, ctx->stream>>>(64, dpart, S.loss);
   T9_CUDA(cudaMemsetAsync(S.g, 0, sizeof(float) * MLP_NPARAM, ctx->stream));
   auto colsum = [&](int N, const float* X, float* out) {
      k_colsum_part<<<COLSUM_BLOCKS, 256, 0, ctx->stream>>>(rows, N, X, S.split);
      k_colsum_final<<<N, COLSUM_BLOCKS, 0, ctx->stream>>>(N, S.split, out);
   };
   // layer 3: dW3 = H2^T dY, db3 = colsum dY, dH2 = dY W3^T
   T9_CHECK(gemm(ctx, true, false, MLP_HID, MLP_OUT_PAD, rows, S.h2, MLP_HID, S.dy, MLP_OUT_PAD, S.g + OFF_W3, ns));
   colsum(MLP_OUT_PAD, S.dyf, S.g + OFF_B3);
   T9_CHECK(gemm(ctx, false, true, rows, MLP_HID, MLP_OUT_PAD, S.dy, MLP_OUT_PAD, wb + BF_W3, MLP_OUT_PAD, S.c, 1));
   k_silu_back<<<grid_for((long long)rows * MLP_HID, 256), 256, 0, ctx->stream>>>(rows * MLP_HID, S.c, S.z2, S.dz,
      S.dzf);
   // layer 2: dW2 = H1^T dZ2, db2, dH1 = dZ2 W2^T
   T9_CHECK(gemm(ctx, true, false, MLP_HID, MLP_HID, rows, S.h1, MLP_HID, S.dz, MLP_HID, S.g + OFF_W2, ns));
   colsum(MLP_HID, S.dzf, S.g + OFF_B2);
   T9_CHECK(gemm(ctx, false, true, rows, MLP_HID, MLP_HID, S.dz, MLP_HID, wb + BF_W2, MLP_HID, S.c, 1));
   k_silu_back<<<grid_for((long long)rows * MLP_HID, 256), 256, 0, ctx->stream>>>(rows * MLP_HID, S.c, S.z1, S.dz,
      S.dzf);
   // layer 1: dW1 = X^T dZ1, db1
   T9_CHECK(gemm(ctx, true, false, MLP_IN, MLP_HID, rows, S.x, MLP_IN, S.dz, MLP_HID, S.g + OFF_W1, ns));
   colsum(MLP_HID, S.dzf, S.g + OFF_B1);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

int mlp_adamw(Context* ctx, float lr, float wd)
{
   MlpState& S = ctx->mlp;
   k_adamw<<<1, 1024, 0, ctx->stream>>>(MLP_NPARAM, lr, 0.9f, 0.999f, 1e-8f, wd, S.step, S.w, S.g, S.m, S.v, S.mask,
      reinterpret_cast<__nv_bfloat16*>(S.wb), S.wb_index);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

}  // namespace t9gb
