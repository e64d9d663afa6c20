// Allocation-free variant of the mutual-field kernel (t9gb_ufield_noalloc).
//
// Some callers cannot call cudaMalloc at the point where they need the
// field: host programs that own every device allocation themselves (a
// plugin must not grow the footprint behind the host's allocator), code that
// runs while a stream is being captured into a CUDA graph (an allocation
// would break the capture), and real-time loops that forbid allocator calls
// after start-up.  This entry point serves them: the caller passes device
// inputs and outputs, and the only working memory is a fixed array in the
// library's own device image.
//
// Scope: the damped (non-Ewald) mutual field -T u for d and p dipoles within
// a cutoff, minimum image in an orthorhombic box or no box, every pair with
// mutual scale 1 (the AMOEBA mutual-11..14 scales; the reference's CUDA
// ufield also runs with an empty uexclude table).  All pairs are visited, so
// the size is capped at T9GB_NOALLOC_MAX_ATOMS.
#include <mutex>

#include "common.cuh"

namespace t9gb {

constexpr int NA_GROUP = 16;

// Working memory: three float4 per atom, (x, y, z, pdamp), (ud, thole),
// (up, 0).  Every GPU that loads the library keeps this array (384 KiB)
// until the process exits.
static __device__ __align__(256) float4 g_noalloc_scratch[3 * T9GB_NOALLOC_MAX_ATOMS];

// Device address of the array, looked up once per device.
static std::mutex g_noalloc_mu;
static float4* g_noalloc_ptr[64] = {nullptr};

static int noalloc_scratch(float4** out)
{
   int dev = 0;
   if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
      return T9GB_NO_DEVICE;
   std::lock_guard<std::mutex> lock(g_noalloc_mu);
   if (!g_noalloc_ptr[dev]) {
      void* p = nullptr;
      if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p)
         return T9GB_CUDA_ERR;
      g_noalloc_ptr[dev] = static_cast<float4*>(p);
   }
   *out = g_noalloc_ptr[dev];
   return T9GB_OK;
}

__global__ void k_noalloc_pack(int n, const float* __restrict__ xyz, const float* __restrict__ pdamp,
   const float* __restrict__ thole, const float* __restrict__ uind, const float* __restrict__ uinp,
   float4* __restrict__ rec)
{
   const int i = blockIdx.x * blockDim.x + threadIdx.x;
   if (i >= n)
      return;
   rec[3 * i] = make_float4(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2], pdamp[i]);
   rec[3 * i + 1] = make_float4(uind[3 * i], uind[3 * i + 1], uind[3 * i + 2], thole[i]);
   rec[3 * i + 2] = make_float4(uinp[3 * i], uinp[3 * i + 1], uinp[3 * i + 2], 0.f);
}

// NA_GROUP lanes per atom i walk j = g, g + 16, ...; fixed-order reduction
__global__ void __launch_bounds__(256) k_noalloc_ufield(int n, float lx, float ly, float lz, float ilx, float ily,
   float ilz, float cut2, const float4* __restrict__ rec, float* __restrict__ field, float* __restrict__ fieldp)
{
   const int tid = blockIdx.x * blockDim.x + threadIdx.x;
   const int i = tid / NA_GROUP, g = tid % NA_GROUP;
   const int nwarp_atoms = (n + 1) / 2 * 2;  // whole warps stay converged for the shuffles
   if (i >= nwarp_atoms)
      return;
   float f[6] = {0, 0, 0, 0, 0, 0};
   if (i < n) {
      const float4 pi = rec[3 * i];
      const float pti = rec[3 * i + 1].w;
      for (int j = g; j < n; j += NA_GROUP) {
         if (j == i)
            continue;
         const float4 pk = rec[3 * j];
         const float dx = image1(pk.x - pi.x, lx, ilx);
         const float dy = image1(pk.y - pi.y, ly, ily);
         const float dz = image1(pk.z - pi.z, lz, ilz);
         const float r2 = dx * dx + dy * dy + dz * dz;
         if (r2 > cut2)
            continue;
         const float4 ud = rec[3 * j + 1];
         const float4 up = rec[3 * j + 2];
         const float invr = rsqrtf(r2);
         const float r = r2 * invr;
         // Thole damping (include/seq/damp.h:8-24) and the damped tensor
         // (include/seq/pair_field.h:333-420, non-Ewald branch, u-scale 1)
         const float pgamma = fminf(pti, ud.w);
         float damp = pi.w * pk.w;
         const float ratio = r * __frcp_rn(damp);
         damp = (damp == 0.f) ? -1.0e16f : -pgamma * ratio * ratio * ratio;
         const float ex = __expf(damp);
         const float rr3 = invr * invr * invr;
         const float b1 = (1.f - ex) * rr3;
         const float b2 = (1.f - ex * (1.f - damp)) * 3.f * rr3 * invr * invr;
         float c = b2 * (dx * ud.x + dy * ud.y + dz * ud.z);
         f[0] += c * dx - b1 * ud.x;
         f[1] += c * dy - b1 * ud.y;
         f[2] += c * dz - b1 * ud.z;
         c = b2 * (dx * up.x + dy * up.y + dz * up.z);
         f[3] += c * dx - b1 * up.x;
         f[4] += c * dy - b1 * up.y;
         f[5] += c * dz - b1 * up.z;
      }
   }
#pragma unroll
   for (int c = 0; c < 6; ++c)
#pragma unroll
      for (int o = NA_GROUP / 2; o > 0; o >>= 1)
         f[c] += __shfl_xor_sync(0xffffffffu, f[c], o);
   if (i < n && g < 3) {
      field[3 * i + g] = g == 0 ? f[0] : (g == 1 ? f[1] : f[2]);
      fieldp[3 * i + g] = g == 0 ? f[3] : (g == 1 ? f[4] : f[5]);
   }
}

}  // namespace t9gb

extern "C" int t9gb_ufield_noalloc(int n, const double* box, double cutoff, const float* xyz, const float* pdamp,
   const float* thole, const float* uind, const float* uinp, float* field, float* fieldp, void* stream)
{
   using namespace t9gb;
   if (n <= 0 || !xyz || !pdamp || !thole || !uind || !uinp || !field || !fieldp || !(cutoff > 0))
      return T9GB_BAD_ARG;
   if (n > T9GB_NOALLOC_MAX_ATOMS)
      return T9GB_TOO_LARGE;
   float4* rec = nullptr;
   int rc = noalloc_scratch(&rec);
   if (rc != T9GB_OK)
      return rc;
   const bool pbc = box && box[0] > 0 && box[1] > 0 && box[2] > 0;
   const float lx = pbc ? (float)box[0] : 0.f, ly = pbc ? (float)box[1] : 0.f, lz = pbc ? (float)box[2] : 0.f;
   const float ilx = pbc ? (float)(1.0 / box[0]) : 0.f, ily = pbc ? (float)(1.0 / box[1]) : 0.f;
   const float ilz = pbc ? (float)(1.0 / box[2]) : 0.f;
   const double c2 = cutoff * cutoff;
   const float cut2 = c2 > 3.0e38 ? 3.0e38f : (float)c2;
   cudaStream_t s = static_cast<cudaStream_t>(stream);
   k_noalloc_pack<<<grid_for(n, 256), 256, 0, s>>>(n, xyz, pdamp, thole, uind, uinp, rec);
   const long long threads = (long long)((n + 1) / 2 * 2) * NA_GROUP;
   k_noalloc_ufield<<<grid_for(threads, 256), 256, 0, s>>>(n, lx, ly, lz, ilx, ily, ilz, cut2, rec, field, fieldp);
   return cudaGetLastError() == cudaSuccess ? T9GB_OK : T9GB_CUDA_ERR;
}
