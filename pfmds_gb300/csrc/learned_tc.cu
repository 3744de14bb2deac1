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

static_assert(NET_FLOATS == PFMD_LEARNED_NET_FLOATS, "the header's network size");
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
// Bounded wait for the mbarrier phase with the given parity: at most `limit`
// polls; false on timeout.
__device__ __forceinline__ bool mbar_wait(unsigned long long* mbar, unsigned int parity, unsigned int limit) {
  const unsigned int a = smem_u32(mbar);
  for (unsigned int it = 0; it < limit; ++it) {
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
                                                   float* e_out, float* g_out, Ctl* ctl, unsigned int wait_limit,
                                                   int stall) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  // the operand tiles want 1024-byte alignment; the launch adds 1024 bytes of slack
  unsigned char* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  TcSmem& S = *reinterpret_cast<TcSmem*>(base);
  const int t = threadIdx.x, w = t >> 5;
  if (block_stop(ctl)) return;
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
    if (t == 0 && !stall) {  // stall (test hook): nothing arrives on the mbarrier
      mma_k64(tmem, aA, b_addr);
      mma_commit(&S.mbar);
    }
    const bool ok = mbar_wait(&S.mbar, phase, wait_limit);
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
      mbar_wait(&S.mbar, phase, wait_limit);
      set_error(ctl, PFMD_E_TIMEOUT, EK_NONE, blockIdx.x, 0, 0);
    }
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 64;" ::"r"(tmem) : "memory");
}

// Polls of an mbarrier wait before it gives up (the test hook may lower it).
static unsigned int wait_limit() { return g_wait_hook.spin_limit ? g_wait_hook.spin_limit : (1u << 24); }

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
  k_mlp_tc<<<grid, TC_ROWS, sizeof(TcSmem) + 1024, s>>>(rows, G, d, net, e, g, ctl, wait_limit(),
                                                        g_wait_hook.stall);
  ++g_kernel_launches;
}


// ---------------------------------------------------------------------------
// training on the tensor cores
// ---------------------------------------------------------------------------
// One persistent CTA of 128 threads per SM walks tiles of 128 rows (thread = row =
// TMEM lane) and computes what k_train computes on the CUDA cores: per row the
// forward pass, its tangent along the force-matching direction U and the backward
// pass of both, as six products with M = 128, N = 64, K = 64 --
//   Z1 = X W1^T, ZD1 = U W1^T      (X carries a 1 in column 48 and W1 the bias b1 there)
//   Z2 = A1 W2^T, ZD2 = AD1 W2^T   (A1 = silu(Z1), AD1 = silu'(Z1) ZD1)
//   WB = B2 W2,  WD = P2 W2        (B2 = w3 silu'(Z2), P2 the energy and force path)
// -- and the weight gradient as two products over the rows (K = 2 x 128: the plain
// and the tangent term side by side) that accumulate in TMEM over all of the CTA's
// tiles:
//   ACC1 += [P1 | Q1] . [X | U]          lane h < 64: dW1 (columns f < 48), db1 (column 48);
//                                         lane 64: the sum of dL/dE, db3 (column 48)
//   ACC2 += [P2 | Q2 ; A3 | 0] . [A1 | AD1]  lane h < 64: dW2, db2 (column 64, A1's 1s);
//                                         lane 64 + h: dw3 (column 64)
// Those operands are stored transposed (K = the tile's rows), in the same no-swizzle
// core-matrix layout with 4 KiB between 8-row groups.  Each CTA writes its partial
// gradient once; k_train_reduce sums the partials in a fixed order, so a run
// repeats bit for bit.  TMEM columns: [0, 128) Z1 | ZD1, [128, 192) ACC1,
// [192, 272) ACC2, [288, 416) Z2 | ZD2, then WB | WD.
constexpr int TR_K = 256;                    // K of the weight-gradient products
constexpr int TR_SBO = TR_K / 8 * 128;       // 4 KiB between 8-row groups
constexpr int TR_A_BYTES = 128 * TR_K * 2;   // 64 KiB
constexpr int TR_B1_BYTES = 64 * TR_K * 2;   // 32 KiB: [X | U]^T, N = 64
constexpr int TR_B2_BYTES = 80 * TR_K * 2;   // 40 KiB: [A1 | AD1]^T, N = 80
constexpr unsigned int COL_Z = 0, COL_ACC1 = 128, COL_ACC2 = 192, COL_Z2 = 288;

struct TrSmem {
  alignas(1024) unsigned char R0[TILE_BYTES_A], R1[TILE_BYTES_A];  // row operands, K = 64
  alignas(1024) unsigned char W1[TILE_BYTES_W], W2[TILE_BYTES_W], W2T[TILE_BYTES_W];
  alignas(1024) unsigned char XU[TR_B1_BYTES];
  alignas(1024) unsigned char TA[TR_A_BYTES];   // A of ACC2, then of ACC1
  alignas(1024) unsigned char TB[TR_B2_BYTES];  // B of ACC2
  float b2[NH], w3[NH];
  float b3;
  double red[128];
  alignas(8) unsigned long long mbar;
  unsigned int tmem_base;
  int timeout;
};

__device__ __forceinline__ int off_tr(int m, int k) {
  return (m >> 3) * TR_SBO + (k >> 3) * 128 + (m & 7) * 16 + (k & 7) * 2;
}
__device__ __forceinline__ void st_tr(unsigned char* tile, int m, int k, float v) {
  *reinterpret_cast<__nv_bfloat16*>(tile + off_tr(m, k)) = __float2bfloat16_rn(v);
}
__device__ __forceinline__ unsigned long long sdesc_sbo(unsigned int addr, unsigned int sbo) {
  unsigned long long d = 0;
  d |= static_cast<unsigned long long>((addr >> 4) & 0x3FFFu);
  d |= static_cast<unsigned long long>((128u >> 4) & 0x3FFFu) << 16;
  d |= static_cast<unsigned long long>((sbo >> 4) & 0x3FFFu) << 32;
  d |= 1ull << 46;
  return d;
}
__device__ __forceinline__ unsigned int idesc_bf16_m128(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<unsigned int>(n >> 3) << 17) | ((TC_ROWS >> 4) << 24);
}
// D[128 x n] (+)= A[128 x K] B[n x K]^T, K = 16 * ksteps; the first step overwrites
// unless acc.
__device__ __forceinline__ void mma_gen(unsigned int tmem, unsigned int a_addr, unsigned int b_addr, unsigned int sbo,
                                        int n, int ksteps, bool acc) {
  const unsigned int id = idesc_bf16_m128(n);
  for (int kk = 0; kk < ksteps; ++kk) {
    const unsigned long long da = sdesc_sbo(a_addr + kk * 256, sbo), db = sdesc_sbo(b_addr + kk * 256, sbo);
    const unsigned int a = (acc || kk > 0) ? 1u : 0u;
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(tmem),
        "l"(da), "l"(db), "r"(id), "r"(a));
  }
}
__device__ __forceinline__ void tmem_ld32(unsigned int taddr, float (&v)[32]) {
  unsigned int r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
      "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ float d2silu_f(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f - s) * (2.f + z * (1.f - 2.f * s));
}
__device__ __forceinline__ void zero16(unsigned char* p) { *reinterpret_cast<uint4*>(p) = make_uint4(0, 0, 0, 0); }

__global__ void __launch_bounds__(128, 1) k_train_tc(int rows, const float* __restrict__ G,
                                                     const float* __restrict__ U, const double* __restrict__ tgt,
                                                     float wE, float wF, const Net* __restrict__ net, float* part,
                                                     double* lpart, Ctl* ctl, unsigned int wait_limit, int stall) {
  extern __shared__ __align__(16) unsigned char smem_raw[];
  unsigned char* base = smem_raw + ((1024u - (smem_u32(smem_raw) & 1023u)) & 1023u);
  TrSmem& S = *reinterpret_cast<TrSmem*>(base);
  const int t = threadIdx.x, w = t >> 5;
  // weights (BF16, core-matrix layout): W1 with b1 in column 48
  for (int i = t; i < TC_N * TC_K; i += blockDim.x) {
    const int n = i / TC_K, k = i % TC_K;
    st_bf16(S.W1, n, k, k < NG ? net->W1[n * NG + k] : (k == NG ? net->b1[n] : 0.f));
    st_bf16(S.W2, n, k, net->W2[n * NH + k]);
    st_bf16(S.W2T, n, k, net->W2[k * NH + n]);
  }
  for (int i = t; i < NH; i += blockDim.x) {
    S.b2[i] = net->b2[i];
    S.w3[i] = net->w3[i];
  }
  // operand rows that no tile writes: XU n = 49..63, TB n = 65..79
  for (int i = t; i < 15 * TR_K / 8; i += blockDim.x) zero16(S.XU + off_tr(49 + i / (TR_K / 8), (i % (TR_K / 8)) * 8));
  for (int i = t; i < 15 * TR_K / 8; i += blockDim.x) zero16(S.TB + off_tr(65 + i / (TR_K / 8), (i % (TR_K / 8)) * 8));
  if (t == 0) {
    S.b3 = net->b3;
    S.timeout = 0;
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&S.mbar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (w == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&S.tmem_base))
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  to_async_proxy();
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  const unsigned int tmem = S.tmem_base;
  const unsigned int tl = tmem + (static_cast<unsigned int>(w * 32) << 16);  // this warp's lanes
  const unsigned int aR0 = smem_u32(S.R0), aR1 = smem_u32(S.R1), aW1 = smem_u32(S.W1), aW2 = smem_u32(S.W2),
                     aW2T = smem_u32(S.W2T), aXU = smem_u32(S.XU), aTA = smem_u32(S.TA), aTB = smem_u32(S.TB);
  unsigned int phase = 0;
  bool acc_started = false;
  double se = 0.0;
  const float inv_rows = 1.f / static_cast<float>(rows);
  const int ntiles = (rows + TC_ROWS - 1) / TC_ROWS;
  // operands visible to the tensor core; thread 0 issues `issue`; everyone waits
  auto run = [&](auto issue) -> bool {
    to_async_proxy();
    tc_before_sync();
    __syncthreads();
    tc_after_sync();
    if (t == 0 && !stall) {  // stall (test hook): nothing arrives on the mbarrier
      issue();
      mma_commit(&S.mbar);
    }
    const bool ok = mbar_wait(&S.mbar, phase, wait_limit);
    phase ^= 1u;
    if (!ok) S.timeout = 1;
    tc_after_sync();
    __syncthreads();
    return S.timeout == 0;
  };
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int row = tile * TC_ROWS + t;
    const bool valid = row < rows;
    // X and U: rows of R0 / R1, columns of [X | U]^T
    for (int k = 0; k < TC_K; ++k) {
      const float x = valid ? (k < NG ? G[(size_t)row * NG + k] : (k == NG ? 1.f : 0.f)) : 0.f;
      const float u = (valid && U && k < NG) ? U[(size_t)row * NG + k] : 0.f;
      st_bf16(S.R0, t, k, x);
      st_bf16(S.R1, t, k, u);
      if (k <= NG) {
        st_tr(S.XU, k, t, x);
        st_tr(S.XU, k, TC_ROWS + t, u);
      }
    }
    if (!run([&] {
          mma_gen(tmem + COL_Z, aR0, aW1, 1024, 64, 4, false);
          mma_gen(tmem + COL_Z + 64, aR1, aW1, 1024, 64, 4, false);
        }))
      break;
    // A1 = silu(Z1), AD1 = silu'(Z1) ZD1: rows of R0 / R1, columns of [A1 | AD1]^T
    for (int h0 = 0; h0 < 64; h0 += 32) {
      float z[32], zd[32];
      tmem_ld32(tl + COL_Z + h0, z);
      tmem_ld32(tl + COL_Z + 64 + h0, zd);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int h = h0 + j;
        const float a1 = silu_f(z[j]), ad1 = dsilu_f(z[j]) * zd[j];
        st_bf16(S.R0, t, h, a1);
        st_bf16(S.R1, t, h, ad1);
        st_tr(S.TB, h, t, a1);
        st_tr(S.TB, h, TC_ROWS + t, ad1);
      }
    }
    st_tr(S.TB, 64, t, valid ? 1.f : 0.f);
    st_tr(S.TB, 64, TC_ROWS + t, 0.f);
    if (!run([&] {
          mma_gen(tmem + COL_Z2, aR0, aW2, 1024, 64, 4, false);
          mma_gen(tmem + COL_Z2 + 64, aR1, aW2, 1024, 64, 4, false);
        }))
      break;
    // the energy and dL/dE, then B2 and P2 (rows of R0 / R1), [P2 | Q2 ; A3 | 0]^T
    float E = S.b3;
    for (int h0 = 0; h0 < 64; h0 += 32) {
      float z[32];
      tmem_ld32(tl + COL_Z2 + h0, z);
#pragma unroll
      for (int j = 0; j < 32; ++j) E += S.w3[h0 + j] * silu_f(z[j] + S.b2[h0 + j]);
    }
    float de = 0.f;
    if (valid) {
      const double err = (double)E - tgt[row];
      de = wE * static_cast<float>(2.0 * err) * inv_rows;
      se += err * err;
    }
    for (int h0 = 0; h0 < 64; h0 += 32) {
      float z[32], zd[32];
      tmem_ld32(tl + COL_Z2 + h0, z);
      tmem_ld32(tl + COL_Z2 + 64 + h0, zd);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int h = h0 + j;
        const float z2 = z[j] + S.b2[h], w3 = S.w3[h];
        const float s2 = dsilu_f(z2), b2v = w3 * s2;
        const float p2 = de * w3 * s2 + wF * w3 * d2silu_f(z2) * zd[j];
        const float a3 = de * silu_f(z2) + wF * s2 * zd[j];
        st_bf16(S.R0, t, h, b2v);
        st_bf16(S.R1, t, h, p2);
        st_tr(S.TA, h, t, p2);
        st_tr(S.TA, h, TC_ROWS + t, wF * b2v);
        st_tr(S.TA, 64 + h, t, a3);
        st_tr(S.TA, 64 + h, TC_ROWS + t, 0.f);
      }
    }
    if (!run([&] {
          mma_gen(tmem + COL_ACC2, aTA, aTB, TR_SBO, 80, TR_K / 16, acc_started);
          mma_gen(tmem + COL_Z2, aR0, aW2T, 1024, 64, 4, false);
          mma_gen(tmem + COL_Z2 + 64, aR1, aW2T, 1024, 64, 4, false);
        }))
      break;
    // P1, Q1 and dL/dE: [P1 | Q1 ; de | 0 ; 0]^T
    for (int h0 = 0; h0 < 64; h0 += 32) {
      float wb[32], wd[32], z[32], zd[32];
      tmem_ld32(tl + COL_Z2 + h0, wb);
      tmem_ld32(tl + COL_Z2 + 64 + h0, wd);
      tmem_ld32(tl + COL_Z + h0, z);
      tmem_ld32(tl + COL_Z + 64 + h0, zd);
#pragma unroll
      for (int j = 0; j < 32; ++j) {
        const int h = h0 + j;
        const float s1 = dsilu_f(z[j]);
        st_tr(S.TA, h, t, s1 * wd[j] + wF * d2silu_f(z[j]) * zd[j] * wb[j]);
        st_tr(S.TA, h, TC_ROWS + t, wF * s1 * wb[j]);
      }
    }
    st_tr(S.TA, 64, t, de);
    st_tr(S.TA, 64, TC_ROWS + t, 0.f);
    for (int i = t; i < 63 * TR_K / 8; i += blockDim.x) zero16(S.TA + off_tr(65 + i / (TR_K / 8), (i % (TR_K / 8)) * 8));
    if (!run([&] { mma_gen(tmem + COL_ACC1, aTA, aXU, TR_SBO, 64, TR_K / 16, acc_started); })) break;
    acc_started = true;
  }
  // this CTA's partial gradient
  const int ob1 = NH * NG, oW2 = ob1 + NH, ob2 = oW2 + NH * NH, ow3 = ob2 + NH, ob3 = ow3 + NH;
  float* out = part + (size_t)blockIdx.x * NET_FLOATS;
  if (S.timeout == 0 && acc_started) {
    float v[64];
    tmem_ld64(tl + COL_ACC1, v);
    if (t < NH) {
      for (int f = 0; f < NG; ++f) out[t * NG + f] = v[f];
      out[ob1 + t] = v[NG];
    } else if (t == NH) {
      out[ob3] = v[NG];
    }
    tmem_ld64(tl + COL_ACC2, v);
    if (t < NH)
      for (int c = 0; c < NH; ++c) out[oW2 + t * NH + c] = v[c];
    tmem_ld64(tl + COL_ACC2 + 64, v);
    if (t < NH)
      out[ob2 + t] = v[0];
    else
      out[ow3 + (t - NH)] = v[0];
  }
  S.red[t] = se;
  __syncthreads();
  if (t == 0) {
    double s = 0.0;
    for (int i = 0; i < 128; ++i) s += S.red[i];
    lpart[blockIdx.x] = s;
  }
  if (S.timeout) {
    if (t == 0) {
      mbar_wait(&S.mbar, phase, wait_limit);
      set_error(ctl, PFMD_E_TIMEOUT, EK_NONE, blockIdx.x, 0, 0);
    }
  }
  tc_before_sync();
  __syncthreads();
  tc_after_sync();
  if (w == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tmem) : "memory");
}

int train_tc_grid(int rows) {
  const int ntiles = (rows + TC_ROWS - 1) / TC_ROWS;
  int dev = 0, sms = 148;
  if (cudaGetDevice(&dev) == cudaSuccess) cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return ntiles < sms ? ntiles : sms;
}

void launch_train_grad_tc(int rows, const float* G, const float* U, const double* target_by_row, float wE, float wF,
                          const Net* net, TrainBuf& T, Ctl* ctl, cudaStream_t s) {
  if (rows <= 0) return;
  static bool attr = false;
  if (!attr) {
    cudaFuncSetAttribute(k_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(sizeof(TrSmem)) + 1024);
    attr = true;
  }
  const int grid = train_tc_grid(rows);
  k_train_tc<<<grid, TC_ROWS, sizeof(TrSmem) + 1024, s>>>(rows, G, U, target_by_row, wE, U ? wF : 0.f, net, T.part,
                                                          T.lpart, ctl, wait_limit(), g_wait_hook.stall);
  ++g_kernel_launches;
  launch_train_reduce(grid, rows, T, s);
}

}  // namespace learned
}  // namespace pfmd
