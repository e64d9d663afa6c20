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
   T9_CUDA(cudaMalloc(&S.ticket, sizeof(int)));
   T9_CUDA(cudaMemset(S.ticket, 0, sizeof(int)));
   T9_CUDA(cudaDeviceGetAttribute(&S.sms, cudaDevAttrMultiProcessorCount, ctx->dev));
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
      S.dyf, S.dz, S.dzf, S.err, S.loss, S.split, S.gpart, S.ticket};
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
// 16 warps per 128 rows.  The row tile and the transposed weights are
// staged in shared memory in the canonical K-major layout without swizzle
// (8-row x 16-byte core matrices; LBO = 128 B between core matrices along K,
// SBO = K / 8 x 128 B between 8-row groups), one thread issues the
// tcgen05.mma instructions (M = 128, K = 16 per instruction, BF16 in, FP32
// accumulated in tensor memory), tcgen05.commit signals an mbarrier, and each
// warp reads 16 columns of its 32 rows back with tcgen05.ld for the bias +
// SiLU epilogue, which writes the next layer's operand tile.  The outputs
// are those of the mma.sync path, equal to them up to the order of the FP32
// accumulation inside the MMA.

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

// the same tile read MN-major (its rows are the K dimension): without
// swizzle the descriptor's SBO is the stride between core matrices along
// M / N (128 B, adjacent 8-column groups) and LBO the stride between 8-row
// groups along K
__device__ __forceinline__ unsigned long long smem_desc_mn(unsigned addr, int width)
{
   const unsigned long long lbo = (unsigned long long)((width >> 3) * 128) >> 4, sbo = 128 >> 4;
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

// 16-byte store of 8 bf16 (round to nearest, as __float2bfloat16)
__device__ __forceinline__ void st_bf8(unsigned char* p, const float* v)
{
   uint4 u;
   unsigned* w = reinterpret_cast<unsigned*>(&u);
#pragma unroll
   for (int i = 0; i < 4; ++i) {
      const __nv_bfloat162 b = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
      w[i] = *reinterpret_cast<const unsigned*>(&b);
   }
   *reinterpret_cast<uint4*>(p) = u;
}

// The BF16 weights (W1 | W2 | W3: 832 16-byte chunks) read in one batch of
// independent loads, then scattered into the operand tiles: transposed,
// (n, k) = W[k][n], at w1t / w2t / w3t (W3^T rows 8-15 zero) for the forward
// products; with w2 / w3 >= 0 also as stored, (n, k) = W[n][k] (W3 columns
// 8-15 zero), for the backward products.
template <int NT>
__device__ __forceinline__ void stage_weights(unsigned char* sm, const __nv_bfloat16* __restrict__ wb, int w1t,
   int w2t, int w3t, int w2, int w3)
{
   constexpr int NCH = BF_END / 8, PER = (NCH + NT - 1) / NT;
   static_assert(BF_END % 8 == 0 && BF_W2 % 8 == 0 && BF_W3 % 8 == 0, "16-byte weight chunks");
   const int tid = threadIdx.x;
   uint4 c[PER];
#pragma unroll
   for (int j = 0; j < PER; ++j) {
      const int q = tid + NT * j;
      c[j] = q < NCH ? __ldg(reinterpret_cast<const uint4*>(wb) + q) : make_uint4(0, 0, 0, 0);
   }
   auto st = [&](int off, int n, int k, int K, __nv_bfloat16 v) {
      *reinterpret_cast<__nv_bfloat16*>(sm + off + kmaj_off(n, k, K)) = v;
   };
#pragma unroll
   for (int j = 0; j < PER; ++j) {
      const int q = tid + NT * j;
      if (q >= NCH)
         break;
      const __nv_bfloat16* v = reinterpret_cast<const __nv_bfloat16*>(&c[j]);
      const int e = 8 * q;
      if (e < BF_W2) {  // W1[i][h0 .. h0 + 7]
         const int i = e / MLP_HID, h0 = e % MLP_HID;
#pragma unroll
         for (int u = 0; u < 8; ++u)
            st(w1t, h0 + u, i, MLP_IN, v[u]);
      } else if (e < BF_W3) {  // W2[a][b0 .. b0 + 7]
         const int a = (e - BF_W2) / MLP_HID, b0 = (e - BF_W2) % MLP_HID;
#pragma unroll
         for (int u = 0; u < 8; ++u)
            st(w2t, b0 + u, a, MLP_HID, v[u]);
         if (w2 >= 0)
            *reinterpret_cast<uint4*>(sm + w2 + kmaj_off(a, b0, MLP_HID)) = c[j];
      } else {  // W3[h][0 .. 7]
         const int h = (e - BF_W3) / MLP_OUT_PAD;
#pragma unroll
         for (int u = 0; u < 8; ++u)
            st(w3t, u, h, MLP_HID, v[u]);
         if (w3 >= 0) {
            *reinterpret_cast<uint4*>(sm + w3 + kmaj_off(h, 0, 16)) = c[j];
            *reinterpret_cast<uint4*>(sm + w3 + kmaj_off(h, 8, 16)) = make_uint4(0, 0, 0, 0);
         }
      }
   }
   for (int e = tid; e < 8 * MLP_HID; e += NT)
      st(w3t, 8 + e / MLP_HID, e % MLP_HID, MLP_HID, __float2bfloat16(0.f));
}

// operand tiles (bytes): X [128][32], H1 / H2 [128][64], W1^T [64][32],
// W2^T [64][64], W3^T [16][64] (columns 8-15 zero)
constexpr int TC_SX = 0, TC_SH1 = TC_SX + 128 * 32 * 2, TC_SH2 = TC_SH1 + 128 * 64 * 2;
constexpr int TC_SW1 = TC_SH2 + 128 * 64 * 2, TC_SW2 = TC_SW1 + 64 * 32 * 2, TC_SW3 = TC_SW2 + 64 * 64 * 2;
constexpr int TC_SMEM = TC_SW3 + 16 * 64 * 2;  // 55,296 bytes: at most four CTAs per SM, 4 x 128 TMEM columns

// inference: stores only y (the training pass recomputes the activations).
// 16 warps: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows) and
// columns 16 (w / 4) .. + 15 of each 64-column accumulator.
constexpr int TC_THREADS = 512;

__global__ void __launch_bounds__(TC_THREADS, 2) k_mlp_forward_tc(int rows, const __nv_bfloat16* __restrict__ x,
   const __nv_bfloat16* __restrict__ wb, const float* __restrict__ w, float* __restrict__ y, int* __restrict__ err)
{
   extern __shared__ __align__(128) unsigned char tsm[];
   __shared__ __align__(8) unsigned long long bar;
   __shared__ unsigned tmem_slot;
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int quad = warp & 3, col = 16 * (warp >> 2);
   const int r0 = blockIdx.x * TC_ROWS;
   const int rl = 32 * quad + lane, r = r0 + rl;  // this thread's row
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
   // operand tiles: the input rows (one 16-byte chunk per thread) and the
   // transposed weights
   {
      const int rr = tid >> 2, ch = tid & 3;
      const uint4 v = r0 + rr < rows ? __ldg(reinterpret_cast<const uint4*>(x + (size_t)(r0 + rr) * MLP_IN) + ch)
                                     : make_uint4(0, 0, 0, 0);
      *reinterpret_cast<uint4*>(tsm + TC_SX + kmaj_off(rr, 8 * ch, MLP_IN)) = v;
   }
   stage_weights<TC_THREADS>(tsm, wb, TC_SW1, TC_SW2, TC_SW3, -1, -1);
   // the tiles (generic proxy) before the tensor core reads them (async proxy)
   asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   const unsigned tmem = tmem_slot;
   const unsigned lane_base = tmem + ((unsigned)(32 * quad) << 16);
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

   // hidden layer epilogue: h = silu(D + b) into the next operand tile
   // (zero past the rows)
   auto hidden = [&](unsigned dcol, const float* b, unsigned h_off) {
      float v[16];
      tc_ld16(lane_base + dcol + col, v);
#pragma unroll
      for (int i = 0; i < 16; ++i)
         v[i] = r < rows ? silu(v[i] + b[col + i]) : 0.f;
      st_bf8(tsm + h_off + kmaj_off(rl, col, MLP_HID), v);
      st_bf8(tsm + h_off + kmaj_off(rl, col + 8, MLP_HID), v + 8);
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   };

   layer(TC_SX, TC_SW1, MLP_IN, MLP_HID, 0);
   hidden(0, w + OFF_B1, TC_SH1);
   layer(TC_SH1, TC_SW2, MLP_HID, MLP_HID, 64);
   hidden(64, w + OFF_B2, TC_SH2);
   layer(TC_SH2, TC_SW3, MLP_HID, 16, 0);
   if (col == 0) {
      float v[16];
      tc_ld16(lane_base, v);
      if (r < rows) {
         float4* yo = reinterpret_cast<float4*>(y + (size_t)r * MLP_OUT_PAD);
         yo[0] = make_float4(v[0] + w[OFF_B3], v[1] + w[OFF_B3 + 1], v[2] + w[OFF_B3 + 2], v[3] + w[OFF_B3 + 3]);
         yo[1] = make_float4(v[4] + w[OFF_B3 + 4], v[5] + w[OFF_B3 + 5], v[6] + w[OFF_B3 + 6], v[7] + w[OFF_B3 + 7]);
      }
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
// Training pass on tcgen05.  A persistent CTA of 16 warps takes 128-row
// tiles (tile = blockIdx.x + k gridDim.x, a fixed assignment) and for each
// one recomputes the forward pass from x alone (no stored activations), then
// the loss gradient dY, the deltas dZ2 = (dY W3^T) silu'(z2) and
// dZ1 = (dZ2 W2^T) silu'(z1), and adds the tile's weight gradients into
// tensor-memory accumulators that live across its tiles:
//     [dW2 . ; . dW3] += [h1 h2]^T [dZ2 dY]   (one 128 x 80 product)
//     [. ; dW1 ; .]   += [dZ1 x 0]^T dZ1       (rows 64-95 are dW1)
// The transposed operands are the row-major tiles themselves, read
// MN-major by the tensor core, so no transposed copies are stored.  The bias
// gradients are column sums of the FP32 deltas (warp halving butterflies,
// then the four row quadrants); the squared error is summed in FP64.  Each CTA
// writes one partial gradient vector; k_grad_sum adds them in a fixed order.
// The BF16 rounding points are those of the mma.sync path: operands and
// deltas rounded for the products, the bias sums and dY kept in FP32.

// shared-memory tiles (bf16, the K-major no-swizzle layout of kmaj_off)
constexpr int TT_Q = 0;                          // [128][128]: dZ1 0-63 | x 64-95 | 0
constexpr int TT_H = TT_Q + 128 * 128 * 2;       // [128][128]: h1 0-63 | h2 64-127
constexpr int TT_G = TT_H + 128 * 128 * 2;       // [128][80]:  dZ2 0-63 | dY 64-71 | 0
constexpr int TT_W1T = TT_G + 128 * 80 * 2;      // [64][32]  (n, k) = W1[k][n]
constexpr int TT_W2T = TT_W1T + 64 * 32 * 2;     // [64][64]  (n, k) = W2[k][n]
constexpr int TT_W3T = TT_W2T + 64 * 64 * 2;     // [16][64]  (n, k) = W3[k][n], rows 8-15 zero
constexpr int TT_W2 = TT_W3T + 16 * 64 * 2;      // [64][64]  (n, k) = W2[n][k]
constexpr int TT_W3 = TT_W2 + 64 * 64 * 2;       // [64][16]  (n, k) = W3[n][k], columns 8-15 zero
constexpr int TT_BIAS = TT_W3 + 64 * 16 * 2;     // b1 | b2 | b3, f32 [136]
constexpr int TT_BP = TT_BIAS + 136 * 4;         // bias-gradient partials, f32 [4 warps][136]
constexpr int TT_END = TT_BP + 4 * 136 * 4;      // 113,312 bytes
static_assert(TT_END == 113312, "training tile layout");
// requested: 116 KB, so that two CTAs never share an SM (each holds 512
// tensor-memory columns, all of an SM's)
constexpr int TT_SMEM = 116 * 1024;
// tensor-memory columns: forward accumulators, the delta product (dH2, then
// dH1 in the same columns once dY W3^T has been read), the gradients
constexpr int TT_C_D1 = 0, TT_C_D2 = 64, TT_C_D3 = 128, TT_C_DH = 128, TT_C_DWS = 192, TT_C_DW1 = 288;
constexpr int TT_TMEM_COLS = 512;

// column sums over the warp's 32 rows of 16 values per lane: four halving
// stages (lane bit 4, 3, 2, 1 keeps the upper or lower half of its values
// and adds its partner's other half), then one butterfly stage; lane L holds
// the sum of column L >> 1
__device__ __forceinline__ float warp_colsum16(float* v, int lane)
{
#pragma unroll
   for (int st = 0; st < 4; ++st) {
      const int d = 16 >> st, h = 8 >> st;
      const bool up = (lane & d) != 0;
#pragma unroll
      for (int i = 0; i < h; ++i) {
         const float send = up ? v[i] : v[i + h];
         const float keep = up ? v[i + h] : v[i];
         v[i] = keep + __shfl_xor_sync(0xffffffffu, send, d);
      }
   }
   return v[0] + __shfl_xor_sync(0xffffffffu, v[0], 1);
}

// the same for 8 values: three halving stages, two butterfly stages; lane L
// holds the sum of column L >> 2
__device__ __forceinline__ float warp_colsum8(float* v, int lane)
{
#pragma unroll
   for (int st = 0; st < 3; ++st) {
      const int d = 16 >> st, h = 4 >> st;
      const bool up = (lane & d) != 0;
#pragma unroll
      for (int i = 0; i < h; ++i) {
         const float send = up ? v[i] : v[i + h];
         const float keep = up ? v[i + h] : v[i];
         v[i] = keep + __shfl_xor_sync(0xffffffffu, send, d);
      }
   }
   float a = v[0];
   a += __shfl_xor_sync(0xffffffffu, a, 2);
   a += __shfl_xor_sync(0xffffffffu, a, 1);
   return a;
}

// 16 warps: warp w reads TMEM lanes 32 (w % 4) .. + 31 (its rows) and
// columns 16 (w / 4) .. + 15 of each 64-column accumulator
constexpr int TT_THREADS = 512;

__global__ void __launch_bounds__(TT_THREADS, 1) k_mlp_train_tc(int rows, int tiles_per_cta, int npad,
   const float* __restrict__ rowpol, const __nv_bfloat16* __restrict__ x, const float* __restrict__ t,
   const __nv_bfloat16* __restrict__ wb, const float* __restrict__ w, float* __restrict__ gpart,
   double* __restrict__ lpart, int* __restrict__ err)
{
   extern __shared__ __align__(128) unsigned char tsm[];
   __shared__ __align__(8) unsigned long long bar;
   __shared__ unsigned tmem_slot;
   __shared__ double lsum[TT_THREADS / 32];
   const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
   const int quad = warp & 3, cg = warp >> 2;  // TMEM lane quadrant, 16-column group
   const int rl = 32 * quad + lane;            // this thread's row of a tile (its TMEM lane)
   const int col = 16 * cg;
   const unsigned base = (unsigned)__cvta_generic_to_shared(tsm);
   const unsigned bar_s = (unsigned)__cvta_generic_to_shared(&bar);
   float* bias = reinterpret_cast<float*>(tsm + TT_BIAS);
   float* bpart = reinterpret_cast<float*>(tsm + TT_BP);  // [quadrant][136]

   if (warp == 0) {
      asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                      (unsigned)__cvta_generic_to_shared(&tmem_slot)),
                   "r"((unsigned)TT_TMEM_COLS)
                   : "memory");
      asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
   }
   if (tid == 0)
      mbar_init(bar_s, 1);
   // weights, biases, cleared partials and the zero columns of Q, once per CTA
   stage_weights<TT_THREADS>(tsm, wb, TT_W1T, TT_W2T, TT_W3T, TT_W2, TT_W3);
   for (int c = tid; c < 136; c += TT_THREADS)
      bias[c] = c < 64 ? w[OFF_B1 + c] : c < 128 ? w[OFF_B2 + c - 64] : w[OFF_B3 + c - 128];
   for (int c = tid; c < 4 * 136; c += TT_THREADS)
      bpart[c] = 0.f;
   *reinterpret_cast<uint4*>(tsm + TT_Q + kmaj_off(tid >> 2, 96 + 8 * (tid & 3), 128)) = make_uint4(0, 0, 0, 0);

   unsigned phase = 0;
   auto sync_tiles = [&]() {
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
      __syncthreads();
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   };
   auto wait = [&]() {
      if (!mbar_wait_bounded(bar_s, phase)) {
         // record it, and give the products in flight a second bounded wait
         // before their operands and accumulators are reused or freed
         if (tid == 0)
            atomicOr(err, 4);
         mbar_wait_bounded(bar_s, phase);
      }
      phase ^= 1u;
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
   };
   sync_tiles();
   const unsigned tmem = tmem_slot;
   const unsigned lane_base = tmem + ((unsigned)(32 * quad) << 16);
   // D[dcol..] (+)= A B over K: A at a_off in a tile of width wa, B at b_off
   // in a tile of width wbw; K-major operands step 16 columns (256 bytes),
   // MN-major ones 16 rows (two 8-row groups)
   auto mmas = [&](int dcol, int a_off, int wa, int b_off, int wbw, int K, int n, bool mn, bool acc) {
      const unsigned idesc = tc_idesc(n) | (mn ? (1u << 15) | (1u << 16) : 0u);
      const int sa = mn ? 2 * (wa / 8) * 128 : 256, sb = mn ? 2 * (wbw / 8) * 128 : 256;
      for (int kk = 0; kk < K / 16; ++kk) {
         const unsigned a = base + a_off + kk * sa, b = base + b_off + kk * sb;
         tc_mma(tmem + dcol, mn ? smem_desc_mn(a, wa) : smem_desc(a, wa), mn ? smem_desc_mn(b, wbw) : smem_desc(b, wbw),
            idesc, acc || kk > 0);
      }
   };
   // hidden layer: h = silu(D + b) into H columns hcol.. (zero past the rows)
   auto hidden = [&](int dcol, const float* b, int hcol, bool in) {
      float v[16];
      tc_ld16(lane_base + dcol + col, v);
#pragma unroll
      for (int i = 0; i < 16; ++i)
         v[i] = in ? silu(v[i] + b[col + i]) : 0.f;
      st_bf8(tsm + TT_H + kmaj_off(rl, hcol + col, 128), v);
      st_bf8(tsm + TT_H + kmaj_off(rl, hcol + col + 8, 128), v + 8);
   };
   // delta: dZ = dH silu'(z), z = D + b re-read from the forward
   // accumulator; BF16 into (off, width) columns 0-63, FP32 column sums
   // into bpart[quad][boff..]
   auto delta = [&](int zcol, const float* b, int off, int width, int boff, bool in) {
      float dh[16], z[16];
      tc_ld16(lane_base + TT_C_DH + col, dh);
      tc_ld16(lane_base + zcol + col, z);
#pragma unroll
      for (int i = 0; i < 16; ++i)
         dh[i] = in ? dh[i] * silu_grad(z[i] + b[col + i]) : 0.f;
      st_bf8(tsm + off + kmaj_off(rl, col, width), dh);
      st_bf8(tsm + off + kmaj_off(rl, col + 8, width), dh + 8);
      const float a = warp_colsum16(dh, lane);
      if ((lane & 1) == 0)
         bpart[quad * 136 + boff + col + (lane >> 1)] += a;
   };

   double se = 0;
   const float dscale = 2.f / (float)(rows * MLP_OUT);
   for (int it = 0; it < tiles_per_cta; ++it) {
      const int r0 = (blockIdx.x + it * gridDim.x) * TC_ROWS;
      if (r0 >= rows)
         break;  // uniform over the CTA
      {  // x rows into Q columns 64-95: one 16-byte chunk per thread, coalesced
         const int rr = tid >> 2, ch = tid & 3;
         uint4 v = make_uint4(0, 0, 0, 0);
         if (r0 + rr < rows)
            v = __ldg(reinterpret_cast<const uint4*>(x + (size_t)(r0 + rr) * MLP_IN) + ch);
         *reinterpret_cast<uint4*>(tsm + TT_Q + kmaj_off(rr, 64 + 8 * ch, 128)) = v;
      }
      const int r = r0 + rl;
      const bool in = r < rows;
      // the loss rows: warps of column group 0
      const bool live = cg == 0 && in && (!rowpol || rowpol[r % npad] != 0.f);
      float tv[MLP_OUT] = {0.f, 0.f, 0.f};
      if (live)
#pragma unroll
         for (int c = 0; c < MLP_OUT; ++c)
            tv[c] = t[(size_t)r * MLP_OUT + c];
      sync_tiles();
      // forward: z1 = x W1 + b1, z2 = h1 W2 + b2, y = h2 W3 + b3
      if (tid == 0) {
         mmas(TT_C_D1, TT_Q + 1024, 128, TT_W1T, MLP_IN, MLP_IN, MLP_HID, false, false);
         tc_commit(bar_s);
      }
      wait();
      hidden(TT_C_D1, bias, 0, in);
      sync_tiles();
      if (tid == 0) {
         mmas(TT_C_D2, TT_H, 128, TT_W2T, MLP_HID, MLP_HID, MLP_HID, false, false);
         tc_commit(bar_s);
      }
      wait();
      hidden(TT_C_D2, bias + 64, 64, in);
      sync_tiles();
      if (tid == 0) {
         mmas(TT_C_D3, TT_H + 1024, 128, TT_W3T, MLP_HID, MLP_HID, 16, false, false);
         tc_commit(bar_s);
      }
      wait();
      // loss gradient (k_loss_grad): dY = 2 (y - t) / (3 rows) on live rows
      if (cg == 0) {
         float v[16], dy[MLP_OUT_PAD];
         tc_ld16(lane_base + TT_C_D3, v);
#pragma unroll
         for (int c = 0; c < MLP_OUT_PAD; ++c) {
            float g = 0.f;
            if (c < MLP_OUT && live) {
               const float d = v[c] + bias[128 + c] - tv[c];
               se += (double)d * d;
               g = dscale * d;
            }
            dy[c] = g;
         }
         st_bf8(tsm + TT_G + kmaj_off(rl, 64, 80), dy);
         *reinterpret_cast<uint4*>(tsm + TT_G + kmaj_off(rl, 72, 80)) = make_uint4(0, 0, 0, 0);
         const float a = warp_colsum8(dy, lane);
         if ((lane & 3) == 0)
            bpart[quad * 136 + 128 + (lane >> 2)] += a;
      }
      sync_tiles();
      // dH2 = dY W3^T
      if (tid == 0) {
         mmas(TT_C_DH, TT_G + 1024, 80, TT_W3, 16, 16, MLP_HID, false, false);
         tc_commit(bar_s);
      }
      wait();
      delta(TT_C_D2, bias + 64, TT_G, 80, 64, in);
      sync_tiles();
      // dH1 = dZ2 W2^T; [dW2 . ; . dW3] += [h1 h2]^T [dZ2 dY]
      if (tid == 0) {
         mmas(TT_C_DH, TT_G, 80, TT_W2, MLP_HID, MLP_HID, MLP_HID, false, false);
         mmas(TT_C_DWS, TT_H, 128, TT_G, 80, TC_ROWS, 80, true, it > 0);
         tc_commit(bar_s);
      }
      wait();
      delta(TT_C_D1, bias, TT_Q, 128, 0, in);
      sync_tiles();
      // rows 64-95 of [dZ1 x 0]^T dZ1 are dW1 = x^T dZ1
      if (tid == 0) {
         mmas(TT_C_DW1, TT_Q, 128, TT_Q, 128, TC_ROWS, MLP_HID, true, it > 0);
         tc_commit(bar_s);
      }
      wait();  // Q is rewritten by the next tile
   }

   // this CTA's gradient vector, in the parameter layout of the master weights
   float* gp = gpart + (size_t)blockIdx.x * MLP_NPARAM;
   {
      float v[16];
      auto put16 = [&](float* dst) {
#pragma unroll
         for (int i = 0; i < 16; i += 4)
            *reinterpret_cast<float4*>(dst + i) = make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]);
      };
      if (quad < 2) {  // lanes 0-63: dW2 rows
         tc_ld16(lane_base + TT_C_DWS + col, v);
         put16(gp + OFF_W2 + rl * MLP_HID + col);
      } else {
         const int h = rl - 64;
         if (cg == 0) {  // lanes 64-127: dW3 rows
            tc_ld16(lane_base + TT_C_DWS + 64, v);
            *reinterpret_cast<float4*>(gp + OFF_W3 + h * MLP_OUT_PAD) = make_float4(v[0], v[1], v[2], v[3]);
            *reinterpret_cast<float4*>(gp + OFF_W3 + h * MLP_OUT_PAD + 4) = make_float4(v[4], v[5], v[6], v[7]);
         }
         if (quad == 2) {  // lanes 64-95: dW1 rows
            tc_ld16(lane_base + TT_C_DW1 + col, v);
            put16(gp + OFF_W1 + h * MLP_HID + col);
         }
      }
   }
   {
      double a = se;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         a += __shfl_xor_sync(0xffffffffu, a, o);
      if (lane == 0)
         lsum[warp] = a;
   }
   asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
   __syncthreads();
   for (int c = tid; c < 136; c += TT_THREADS) {
      const float a = (bpart[c] + bpart[136 + c]) + (bpart[272 + c] + bpart[408 + c]);
      gp[c < 64 ? OFF_B1 + c : c < 128 ? OFF_B2 + c - 64 : OFF_B3 + c - 128] = a;
   }
   if (tid == 0)  // the loss rows are in warps 0-3
      lpart[blockIdx.x] = (lsum[0] + lsum[1]) + (lsum[2] + lsum[3]);
   if (warp == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
      asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"((unsigned)TT_TMEM_COLS)
                   : "memory");
   }
}

int mlp_tc_setup()
{
   return cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TT_SMEM) ==
            cudaSuccess &&
         cudaFuncSetAttribute(k_mlp_forward_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, TC_SMEM) == cudaSuccess
      ? T9GB_OK
      : T9GB_CUDA_ERR;
}

// Fixed-order sum of the per-CTA partial gradients: a block takes 32
// parameters, its eight warps stride over the partials, and the eight warp
// sums combine in a fixed tree.  ADAM: the AdamW step (as k_adamw) follows
// in the same thread; the step count is read by every block and advanced by
// the last one.  Block 0 sums the squared errors; scal (may be null) takes
// them times loss_norm.
template <bool ADAM>
__global__ void __launch_bounds__(256) k_grad_sum(int ncta, const float* __restrict__ gpart,
   const double* __restrict__ lpart, const unsigned char* __restrict__ mask, float* __restrict__ g,
   double* __restrict__ loss, double* __restrict__ scal, double loss_norm, float lr, float wd,
   int* __restrict__ step, int* __restrict__ ticket, float* __restrict__ w, float* __restrict__ m,
   float* __restrict__ v, __nv_bfloat16* __restrict__ wb, const int* __restrict__ wb_index)
{
   __shared__ float sh[8][33];
   const int pl = threadIdx.x & 31, sl = threadIdx.x >> 5;
   const int p = blockIdx.x * 32 + pl;
   const int t = ADAM ? *step + 1 : 0;
   // eight independent loads in flight per step (a dependent chain of
   // global loads would pay the latency per partial)
   float a = 0.f;
   if (p < MLP_NPARAM)
      for (int c0 = sl; c0 < ncta; c0 += 64) {
         float u[8];
#pragma unroll
         for (int k = 0; k < 8; ++k) {
            const int c = c0 + 8 * k;
            u[k] = c < ncta ? gpart[(size_t)c * MLP_NPARAM + p] : 0.f;
         }
#pragma unroll
         for (int k = 0; k < 8; ++k)
            a += u[k];
      }
   sh[sl][pl] = a;
   __syncthreads();
   if (sl == 0 && p < MLP_NPARAM) {
      const float gi =
         mask[p] ? ((sh[0][pl] + sh[1][pl]) + (sh[2][pl] + sh[3][pl])) + ((sh[4][pl] + sh[5][pl]) + (sh[6][pl] + sh[7][pl]))
                 : 0.f;
      g[p] = gi;
      if (ADAM && mask[p]) {
         const float beta1 = 0.9f, beta2 = 0.999f, eps = 1e-8f;
         const float c1 = 1.f - powf(beta1, (float)t), c2 = 1.f - powf(beta2, (float)t);
         const float mi = beta1 * m[p] + (1.f - beta1) * gi;
         const float vi = beta2 * v[p] + (1.f - beta2) * gi * gi;
         m[p] = mi;
         v[p] = vi;
         float wi = w[p];
         wi -= lr * ((mi / c1) / (sqrtf(vi / c2) + eps) + wd * wi);
         w[p] = wi;
         if (wb_index[p] >= 0)
            wb[wb_index[p]] = __float2bfloat16(wi);
      }
   }
   if (blockIdx.x == 0 && sl == 1) {  // the squared errors: lane strides, then a fixed butterfly
      double l = 0;
      for (int c = pl; c < ncta; c += 32)
         l += lpart[c];
#pragma unroll
      for (int o = 16; o > 0; o >>= 1)
         l += __shfl_xor_sync(0xffffffffu, l, o);
      if (pl == 0) {
         *loss = l;
         if (scal)
            *scal = l * loss_norm;
      }
   }
   if (ADAM) {
      __shared__ bool last;
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0)
         last = atomicAdd(ticket, 1) == (int)gridDim.x - 1;
      __syncthreads();
      if (last && threadIdx.x == 0) {
         *step = t;
         *ticket = 0;
      }
   }
}

// forward over rows of S.x; outputs in S.y [rows][8] (the mma.sync path
// also keeps the activations its backward pass reads)
int mlp_forward(Context* ctx, int rows)
{
   MlpState& S = ctx->mlp;
   const __nv_bfloat16* wb = reinterpret_cast<const __nv_bfloat16*>(S.wb);
   if (ctx->mlp_tc) {
      k_mlp_forward_tc<<<grid_for(rows, TC_ROWS), TC_THREADS, TC_SMEM, ctx->stream>>>(rows, S.x, wb, S.w, S.y,
         ctx->copy_err);
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

// the tcgen05 training pass over rows of S.x with targets S.t, then the
// gradient sum (ADAM: and the AdamW step; scal: the loss times loss_norm)
static int train_tc(Context* ctx, int rows, const float* rowpol, int npad, bool adam, float lr, float wd,
   double* scal, double loss_norm)
{
   MlpState& S = ctx->mlp;
   const int tiles = (rows + TC_ROWS - 1) / TC_ROWS;
   const int per = (tiles + S.sms - 1) / S.sms;
   const int grid = (tiles + per - 1) / per;
   k_mlp_train_tc<<<grid, TT_THREADS, TT_SMEM, ctx->stream>>>(rows, per, npad, rowpol, S.x, S.t,
      reinterpret_cast<const __nv_bfloat16*>(S.wb), S.w, S.gpart, S.err, ctx->copy_err);
   auto k = adam ? k_grad_sum<true> : k_grad_sum<false>;
   k<<<(MLP_NPARAM + 31) / 32, 256, 0, ctx->stream>>>(grid, S.gpart, S.err, S.mask, S.g, S.loss, scal, loss_norm, lr,
      wd, S.step, S.ticket, S.w, S.m, S.v, reinterpret_cast<__nv_bfloat16*>(S.wb), S.wb_index);
   T9_CUDA(cudaGetLastError());
   return T9GB_OK;
}

// loss and full gradient for rows of S.x with targets S.t: gradient in S.g,
// summed squared error in S.loss.  rowpol (may be null): rows r with
// rowpol[r % npad] == 0 are left out.  The mma.sync path reads the
// activations of the last mlp_forward; the tcgen05 path recomputes them.
int mlp_backward(Context* ctx, int rows, const float* rowpol, int npad)
{
   MlpState& S = ctx->mlp;
   const __nv_bfloat16* wb = reinterpret_cast<const __nv_bfloat16*>(S.wb);
   if (ctx->mlp_tc)
      return train_tc(ctx, rows, rowpol, npad, false, 0.f, 0.f, nullptr, 0.0);
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

int mlp_train_step_tc(Context* ctx, int rows, const float* rowpol, int npad, float lr, float wd, double* scal,
   double loss_norm)
{
   return train_tc(ctx, rows, rowpol, npad, true, lr, wd, scal, loss_norm);
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
