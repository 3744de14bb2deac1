// Learned form, network on the tensor cores: BF16 weights and activations, FP32
// accumulation in tensor memory (tcgen05).
//
// One CTA of 128 threads owns a tile of 128 descriptor rows (one row per thread,
// i.e. one TMEM lane per row).  The four matrix products of a row's energy and
// its gradient dE/dG run as tcgen05.mma kind::f16 with M = 128, N = 64, K = 64
// (four K = 16 steps each), one thread issuing, into one 64-column TMEM
// accumulator that every thread reads back with tcgen05.ld.32x32b.x64:
//   Z1 = Gn W1^T      (+ b1, a1 = silu)
//   Z2 = A1 W2^T      (+ b2, a2 = silu, E = w3 . a2 + b3, e2 = w3 silu'(Z2))
//   T1 = E2 W2        (e1 = T1 silu'(Z1))
//   GH = E1 W1        (dE/dG = GH * inv_std)
// The element-wise steps run in FP32 registers between the products.  Shared
// memory operands use the no-swizzle K-major layout of 8-row x 16-byte core
// matrices: element (r, k) of a tile lives at (r/8)*1024 + (k/8)*128 + (r%8)*16 +
// (k%8)*2 bytes, so neighbouring core matrices are 128 B apart along K (leading
// byte offset) and 1024 B apart along M/N (stride byte offset).  The descriptor
// dimension (48) is padded to 64 with zeros.  MMA completion is signalled through
// an mbarrier; every wait on it is bounded and records a timeout in the status
// block instead of spinning on.
#include <cuda_bf16.h>

#include <cstdint>

#include "../../include/pfmd.h"
#include "forces.cuh"
#include "learned.h"

namespace pfmd {
namespace learned {

constexpr int TC_ROWS = 128, TC_K = 64, TC_N = 64;
constexpr int TILE_BYTES_A = TC_ROWS * TC_K * 2;  // 16 KiB
constexpr int TILE_BYTES_W = TC_N * TC_K * 2;     // 8 KiB

struct TcSmem {
  alignas(1024) unsigned char A[TILE_BYTES_A];
  alignas(1024) unsigned char W1[TILE_BYTES_W], W2[TILE_BYTES_W], W2T[TILE_BYTES_W], W1T[TILE_BYTES_W];
  float b1[NH], b2[NH], w3[NH], inv_std[NG], mean[NG];
  float b3;
  alignas(8) unsigned long long mbar;
  unsigned int tmem_base;
  int timeout;
};

__device__ __forceinline__ unsigned int smem_u32(const void* p) {
  return static_cast<unsigned int>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ int core_off(int r, int k) {
  return (r >> 3) * 1024 + (k >> 3) * 128 + (r & 7) * 16 + (k & 7) * 2;
}
__device__ __forceinline__ void st_bf16(unsigned char* tile, int r, int k, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + core_off(r, k)) = __float2bfloat16_rn(v);
}

// tcgen05 shared-memory matrix descriptor: start address, leading / stride byte
// offsets (>> 4), version 1, no swizzle.
__device__ __forceinline__ unsigned long long sdesc(unsigned int addr) {
  unsigned long long d = 0;
  d |= static_cast<unsigned long long>((addr >> 4) & 0x3FFFu);
  d |= static_cast<unsigned long long>((128u >> 4) & 0x3FFFu) << 16;   // leading byte offset: next core along K
  d |= static_cast<unsigned long long>((1024u >> 4) & 0x3FFFu) << 32;  // stride byte offset: next 8 rows
  d |= 1ull << 46;                                                       // descriptor version
  return d;                                                              // layout type 0: no swizzle
}
// Instruction descriptor, kind::f16: D F32, A and B BF16, both K-major, N = 64, M = 128.
__device__ __forceinline__ unsigned int idesc_bf16_m128_n64() {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((TC_N >> 3) << 17) | ((TC_ROWS >> 4) << 24);
}

__device__ __forceinline__ void mma_k64(unsigned int tmem, unsigned int a_addr, unsigned int b_addr) {
  const unsigned int id = idesc_bf16_m128_n64();
#pragma unroll
  for (int kk = 0; kk < TC_K / 16; ++kk) {
    const unsigned long long da = sdesc(a_addr + kk * 256), db = sdesc(b_addr + kk * 256);
    const unsigned int acc = kk > 0 ? 1u : 0u;
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(id), "r"(acc));
  }
}
__device__ __forceinline__ void mma_commit(unsigned long long* mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(mbar))
               : "memory");
}
// Bounded wait for the mbarrier phase with the given parity; false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned long long* mbar, unsigned int parity) {
  const unsigned int a = smem_u32(mbar);
  for (unsigned int it = 0; it < (1u << 24); ++it) {
    unsigned int done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(a), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}
__device__ __forceinline__ void tmem_ld64(unsigned int taddr, float (&v)[64]) {
  unsigned int r[64];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x64.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31, %32, %33, %34, %35, "
      "%36, %37, %38, %39, %40, %41, %42, %43, %44, %45, %46, %47, %48, %49, %50, %51, %52, %53, %54, %55, %56, "
      "%57, %58, %59, %60, %61, %62, %63}, [%64];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31]),
        "=r"(r[32]), "=r"(r[33]), "=r"(r[34]), "=r"(r[35]), "=r"(r[36]), "=r"(r[37]), "=r"(r[38]), "=r"(r[39]),
        "=r"(r[40]), "=r"(r[41]), "=r"(r[42]), "=r"(r[43]), "=r"(r[44]), "=r"(r[45]), "=r"(r[46]), "=r"(r[47]),
        "=r"(r[48]), "=r"(r[49]), "=r"(r[50]), "=r"(r[51]), "=r"(r[52]), "=r"(r[53]), "=r"(r[54]), "=r"(r[55]),
        "=r"(r[56]), "=r"(r[57]), "=r"(r[58]), "=r"(r[59]), "=r"(r[60]), "=r"(r[61]), "=r"(r[62]), "=r"(r[63])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 64; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ void to_async_proxy() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}
__device__ __forceinline__ void tc_before_sync() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_after_sync() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

__global__ void __launch_bounds__(128, 1) k_mlp_tc(int rows, const float* __restrict__ G,
                                                   const DescPar* __restrict__ Dp, const Net* __restrict__ net,
                                                   float* e_out, float* g_out, Ctl* ctl) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // the operand tiles want 1024-byte alignment; the launch adds 1024 bytes of slack
  unsigned char* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  TcSmem& S = *reinterpret_cast<TcSmem*>(base);
  const int t = threadIdx.x, w = t >> 5;
  if (ctl->stop) return;
  // weights into the core-matrix layout (BF16), padded K / N to 64
  for (int i = t; i < TC_N * TC_K; i += blockDim.x) {
    const int n = i / TC_K, k = i % TC_K;
    st_bf16(S.W1, n, k, k < NG ? net->W1[n * NG + k] : 0.f);                  // B of Z1: [h][f]
    st_bf16(S.W2, n, k, net->W2[n * NH + k]);                                 // B of Z2: [h][c]
    st_bf16(S.W2T, n, k, net->W2[k * NH + n]);                                // B of T1: [c][h]
    st_bf16(S.W1T, n, k, n < NG ? net->W1[k * NG + n] : 0.f);                 // B of GH: [f][c]
  }
  for (int i = t; i < NH; i += blockDim.x) {
    S.b1[i] = net->b1[i];
    S.b2[i] = net->b2[i];
    S.w3[i] = net->w3[i];
  }
  for (int i = t; i < NG; i += blockDim.x) S.inv_std[i] = Dp->inv_std[i];
  if (t == 0) {
    S.b3 = net->b3;
    S.timeout = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 64;" ::"r"(smem_u32(&S.tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  to_async_proxy();
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const unsigned int tmem = S.tmem_base;
  const unsigned int tl = tmem + (static_cast<unsigned int>(w * 32) << 16);  // this warp's 32 lanes
  const unsigned int aA = smem_u32(S.A), aW1 = smem_u32(S.W1), aW2 = smem_u32(S.W2), aW2T = smem_u32(S.W2T),
                     aW1T = smem_u32(S.W1T);
  unsigned int phase = 0;
  const int ntiles = (rows + TC_ROWS - 1) / TC_ROWS;
  // one product: operands in shared memory are visible to the tensor core, thread 0
  // issues, everyone waits and loads its row of the accumulator
  auto product = [&](unsigned int b_addr, float (&v)[64]) -> bool {
    to_async_proxy();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (t == 0) {
      mma_k64(tmem, aA, b_addr);
      mma_commit(&S.mbar);
    }
    const bool ok = mbar_wait(&S.mbar, phase);
    phase ^= 1u;
    if (!ok) S.timeout = 1;
    tc_after_sync();
    tmem_ld64(tl, v);
    tc_before_sync();
    __syncthreads();
    return S.timeout == 0;
  };
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int row = tile * TC_ROWS + t;
    const bool valid = row < rows;
    for (int k = 0; k < TC_K; ++k)
      st_bf16(S.A, t, k, (valid && k < NG) ? G[(size_t)row * NG + k] : 0.f);
    float z1[64], v[64];
    if (!product(aW1, z1)) break;
#pragma unroll
    for (int h = 0; h < 64; ++h) {
      z1[h] += S.b1[h];
      st_bf16(S.A, t, h, silu_f(z1[h]));
    }
    if (!product(aW2, v)) break;
    float E = S.b3;
#pragma unroll
    for (int h = 0; h < 64; ++h) {
      const float z2 = v[h] + S.b2[h];
      E += S.w3[h] * silu_f(z2);
      st_bf16(S.A, t, h, S.w3[h] * dsilu_f(z2));
    }
    if (!product(aW2T, v)) break;
#pragma unroll
    for (int c = 0; c < 64; ++c) st_bf16(S.A, t, c, v[c] * dsilu_f(z1[c]));
    if (!product(aW1T, v)) break;
    if (valid) {
      e_out[row] = E;
#pragma unroll
      for (int f = 0; f < NG; ++f) g_out[(size_t)row * NG + f] = v[f] * S.inv_std[f];
    }
  }
  if (S.timeout) {
    // a product that did not complete in time: give it one more bounded wait before
    // the accumulator is released
    if (t == 0) {
      mbar_wait(&S.mbar, phase);
      set_error(ctl, PFMD_E_TIMEOUT, EK_NONE, blockIdx.x, 0, 0);
    }
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
}

void launch_mlp_tc(int rows, const float* G, const DescPar* d, const Net* net, float* e, float* g, Ctl* ctl,
                   cudaStream_t s) {
  if (rows <= 0) return;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_mlp_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(sizeof(TcSmem)) + 1024);
    attr = true;
  }
  const int ntiles = (rows + TC_ROWS - 1) / TC_ROWS;
  const int grid = ntiles < 148 * 2 ? ntiles : 148 * 2;
  k_mlp_tc<<<grid, TC_ROWS, sizeof(TcSmem) + 1024, s>>>(rows, G, d, net, e, g, ctl);
  ++g_kernel_launches;
}

}  // namespace learned
}  // namespace pfmd
