// mlp_kernels.cu -- learned multidirect-forcing correction.
//
// A per-Lagrangian-point MLP 96 -> 128 -> 128 -> 3 (tanh-form GELU) predicts
// the rest of the multidirect forcing after the first pass: from the slip
// left by pass 0 and the local velocity field it returns dF*dt, the
// velocity-unit correction that the plain passes 1 and 2 would add
// (interp_spread.f90 / forcing.f90, Nl = 3).
//
// Training (forward, backward, weight gradients) runs on the tcgen05 tensor
// cores with TMEM accumulators, one CTA per 128-row tile of the batch, and a
// second kernel sums the tiles' gradients and applies Adam to the FP32
// master weights and their BF16 copies.  Inference in the learned loop is
// the tcgen05 kernel fused with the feature formation; an mma.sync m16n8k16
// inference kernel with the training's rounding points is kept as a check.
//
// Parameter vector (FP32): W1[128][96], b1[128], W2[128][128], b2[128],
// W3[3][128], b3[3].
#include <cuda_bf16.h>
#include <cuda_fp16.h>

#include "kernels.cuh"

namespace ibmk {

typedef __nv_bfloat16 bf16;

// ---- tensor-core fragment helpers (PTX ISA, mma.m16n8k16 .bf16) -----------
__device__ __forceinline__ void mma16816(float c[4], const uint32_t a[4], const uint32_t b[2]) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};\n"
      : "+f"(c[0]), "+f"(c[1]), "+f"(c[2]), "+f"(c[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}
// A tile row-major in shared memory (row stride lda, bf16 elements):
// fragment of rows m0..m0+15, columns k0..k0+15
__device__ __forceinline__ void load_a(uint32_t a[4], const bf16 *As, int lda, int m0, int k0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  a[0] = *reinterpret_cast<const uint32_t *>(&As[(m0 + g) * lda + k0 + 2 * t]);
  a[1] = *reinterpret_cast<const uint32_t *>(&As[(m0 + g + 8) * lda + k0 + 2 * t]);
  a[2] = *reinterpret_cast<const uint32_t *>(&As[(m0 + g) * lda + k0 + 2 * t + 8]);
  a[3] = *reinterpret_cast<const uint32_t *>(&As[(m0 + g + 8) * lda + k0 + 2 * t + 8]);
}
// B operand stored n-major (Bs[n][k], k contiguous, stride ldb)
__device__ __forceinline__ void load_b(uint32_t b[2], const bf16 *Bs, int ldb, int n0, int k0, int lane) {
  const int g = lane >> 2, t = lane & 3;
  b[0] = *reinterpret_cast<const uint32_t *>(&Bs[(n0 + g) * ldb + k0 + 2 * t]);
  b[1] = *reinterpret_cast<const uint32_t *>(&Bs[(n0 + g) * ldb + k0 + 2 * t + 8]);
}

// tanh-form GELU written with the logistic function: 0.5 z (1 + tanh u) =
// z * sigma(2u), u = c (z + a z^3) (the same function; no cancellation for
// negative z, two fast special-function operations instead of tanhf)
// B fragments of two adjacent 8-column tiles (n0..n0+15, k0..k0+15) from
// an n-major shared array by one ldmatrix.x4: b0 = tile n0, b1 = tile n0+8
__device__ __forceinline__ void load_b2(uint32_t b0[2], uint32_t b1[2], const bf16 *Bs, int ldb, int n0, int k0,
                                        int lane) {
  const int m = lane >> 3, i = lane & 7;
  const bf16 *row = Bs + (n0 + (m >> 1) * 8 + i) * ldb + k0 + (m & 1) * 8;
  const uint32_t addr = (uint32_t)__cvta_generic_to_shared(row);
  asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];\n"
               : "=r"(b0[0]), "=r"(b0[1]), "=r"(b1[0]), "=r"(b1[1])
               : "r"(addr));
}
__device__ __forceinline__ float sig2u(float z) {
  const float c = 0.7978845608028654f, a = 0.044715f;
  const float u = c * (z + a * z * z * z);
  return __fdividef(1.f, 1.f + __expf(-2.f * u));
}
__device__ __forceinline__ float gelu_f(float z) { return z * sig2u(z); }
// the same GELU as 0.5 z (1 + tanh(u)) with the hardware tanh (one special-
// function op instead of exp + reciprocal); its error (relative 2^-11 in
// tanh) is below the BF16 rounding of the hidden activations that follows
__device__ __forceinline__ float tanh_hw(float x) {
  float y;
  asm("tanh.approx.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}
__device__ __forceinline__ float gelu_hw(float z) {
  const float c = 0.7978845608028654f, a = 0.044715f;
  const float u = c * (z + a * z * z * z);
  return z * fmaf(0.5f, tanh_hw(u), 0.5f);
}
// d/dz: sigma + z * 2 sigma (1 - sigma) * c (1 + 3 a z^2)
__device__ __forceinline__ float gelu_grad_f(float z) {
  const float c = 0.7978845608028654f, a = 0.044715f;
  const float sg = sig2u(z);
  return sg + 2.f * z * sg * (1.f - sg) * c * (1.f + 3.f * a * z * z);
}

constexpr int NIN = 96, NH = 128, NOUT = 3;
constexpr int LDX = NIN + 8, LDH = NH + 8;  // padded shared-memory rows
constexpr int OFF_B1 = NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH,
              OFF_B3 = OFF_W3 + NOUT * NH, NPARAM = OFF_B3 + NOUT;

// ---------------------------------------------------------------------------
// Inference: X (N x 96, bf16) -> Y (N x 3, fp32), one warp per 16-row tile.
// The layer-1 accumulators become the A fragments of layer 2 in registers:
// the m16n8k16 C fragment of the 8-column tiles 2m and 2m+1 holds exactly the
// A fragment of the 16-column k-block m (rows g, g+8; columns 2t, 2t+1 and
// 2t+8, 2t+9).  Layer 3 is a per-lane partial dot product over the 32
// columns a lane holds, summed over the 4 lanes of a row pair by shuffles.
// Same rounding points as the training's forward pass: BF16 inputs, weights
// of layers 1-2 and hidden activations; FP32 accumulation; FP32 W3.
// ---------------------------------------------------------------------------
constexpr int IW = 12;  // warps per CTA (163 registers: one CTA per SM)
__device__ __forceinline__ uint32_t pack_bf2(float lo, float hi) {
  __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t *>(&v);
}
__global__ void __launch_bounds__(IW * 32, 1) k_mlp_infer(const bf16 *__restrict__ x, int n,
                                                          const bf16 *__restrict__ w1b, const bf16 *__restrict__ w2b,
                                                          const float *__restrict__ params, float *__restrict__ y) {
  extern __shared__ __align__(16) unsigned char sm[];
  bf16 *W1s = reinterpret_cast<bf16 *>(sm);  // [128][LDX]
  bf16 *W2s = W1s + NH * LDX;                // [128][LDH]
  bf16 *Xs = W2s + NH * LDH;                 // [IW][16][LDX]
  float *cst = reinterpret_cast<float *>(Xs + IW * 16 * LDX);  // b1, b2, W3, b3
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int t = tid; t < NH * NIN / 8; t += blockDim.x) {
    const int r = t / (NIN / 8), c8 = (t % (NIN / 8)) * 8;
    *reinterpret_cast<uint4 *>(&W1s[r * LDX + c8]) = *reinterpret_cast<const uint4 *>(&w1b[r * NIN + c8]);
  }
  for (int t = tid; t < NH * NH / 8; t += blockDim.x) {
    const int r = t / (NH / 8), c8 = (t % (NH / 8)) * 8;
    *reinterpret_cast<uint4 *>(&W2s[r * LDH + c8]) = *reinterpret_cast<const uint4 *>(&w2b[r * NH + c8]);
  }
  for (int t = tid; t < NH; t += blockDim.x) { cst[t] = params[OFF_B1 + t]; cst[NH + t] = params[OFF_B2 + t]; }
  for (int t = tid; t < NOUT * NH + NOUT; t += blockDim.x) cst[2 * NH + t] = params[OFF_W3 + t];
  __syncthreads();
  const float *b1 = cst, *b2 = cst + NH, *w3 = cst + 2 * NH, *b3 = w3 + NOUT * NH;
  bf16 *Xw = Xs + warp * 16 * LDX;
  const int g = lane >> 2, tq = lane & 3;
  const int ntiles = (n + 15) / 16;
  for (int tile = blockIdx.x * IW + warp; tile < ntiles; tile += gridDim.x * IW) {
    const long row0 = (long)tile * 16;
    // stage the warp's 16 feature rows (12 x 16 B per row)
    for (int q = lane; q < 16 * (NIN / 8); q += 32) {
      const int r = q / (NIN / 8), c8 = (q % (NIN / 8)) * 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (row0 + r < n) v = __ldg(reinterpret_cast<const uint4 *>(&x[(row0 + r) * NIN + c8]));
      *reinterpret_cast<uint4 *>(&Xw[r * LDX + c8]) = v;
    }
    __syncwarp();
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < NIN; k0 += 16) {
      uint32_t a[4];
      load_a(a, Xw, LDX, 0, k0, lane);
#pragma unroll
      for (int j = 0; j < 16; j += 2) {
        uint32_t b0[2], b1[2];
        load_b2(b0, b1, W1s, LDX, j * 8, k0, lane);
        mma16816(acc[j], a, b0);
        mma16816(acc[j + 1], a, b1);
      }
    }
    // bias + GELU, rounded to BF16 straight into the layer-2 A fragments
    uint32_t af[8][4];
#pragma unroll
    for (int m = 0; m < 8; ++m) {
      const int c0 = 16 * m + 2 * tq, c1 = c0 + 8;
      const float2 p0 = *reinterpret_cast<const float2 *>(&b1[c0]), p1 = *reinterpret_cast<const float2 *>(&b1[c1]);
      af[m][0] = pack_bf2(gelu_f(acc[2 * m][0] + p0.x), gelu_f(acc[2 * m][1] + p0.y));
      af[m][1] = pack_bf2(gelu_f(acc[2 * m][2] + p0.x), gelu_f(acc[2 * m][3] + p0.y));
      af[m][2] = pack_bf2(gelu_f(acc[2 * m + 1][0] + p1.x), gelu_f(acc[2 * m + 1][1] + p1.y));
      af[m][3] = pack_bf2(gelu_f(acc[2 * m + 1][2] + p1.x), gelu_f(acc[2 * m + 1][3] + p1.y));
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
    for (int m = 0; m < 8; ++m) {
#pragma unroll
      for (int j = 0; j < 16; j += 2) {
        uint32_t b0[2], b1[2];
        load_b2(b0, b1, W2s, LDH, j * 8, 16 * m, lane);
        mma16816(acc[j], af[m], b0);
        mma16816(acc[j + 1], af[m], b1);
      }
    }
    // bias + GELU (BF16-rounded), layer 3 partial sums for rows g and g+8
    float part[2][NOUT];
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int o = 0; o < NOUT; ++o) part[h][o] = 0.f;
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int col = j * 8 + 2 * tq;
      const float2 bb = *reinterpret_cast<const float2 *>(&b2[col]);
      float2 w[NOUT];
#pragma unroll
      for (int o = 0; o < NOUT; ++o) w[o] = *reinterpret_cast<const float2 *>(&w3[o * NH + col]);
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const float h0 = __bfloat162float(__float2bfloat16(gelu_f(acc[j][2 * h] + bb.x)));
        const float h1 = __bfloat162float(__float2bfloat16(gelu_f(acc[j][2 * h + 1] + bb.y)));
#pragma unroll
        for (int o = 0; o < NOUT; ++o) part[h][o] += h0 * w[o].x + h1 * w[o].y;
      }
    }
#pragma unroll
    for (int h = 0; h < 2; ++h)
#pragma unroll
      for (int o = 0; o < NOUT; ++o) {
        part[h][o] += __shfl_xor_sync(0xffffffffu, part[h][o], 1);
        part[h][o] += __shfl_xor_sync(0xffffffffu, part[h][o], 2);
      }
    if (tq == 0) {
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const long r = row0 + g + 8 * h;
        if (r < n)
          for (int o = 0; o < NOUT; ++o) y[r * NOUT + o] = part[h][o] + b3[o];
      }
    }
    __syncwarp();
  }
}
size_t mlp_infer_smem() {
  return (size_t)(NH * LDX + NH * LDH + IW * 16 * LDX) * sizeof(bf16) + (size_t)(2 * NH + NOUT * NH + NOUT) * sizeof(float);
}
void launch_mlp_infer(cudaStream_t s, const bf16 *x, int n, const bf16 *w1b, const bf16 *w2b, const float *params,
                      float *y) {
  if (n <= 0) return;
  const int ntiles = (n + 15) / 16;
  const int grid = (ntiles + IW - 1) / IW < 152 ? (ntiles + IW - 1) / IW : 152;
  k_mlp_infer<<<grid, IW * 32, mlp_infer_smem(), s>>>(x, n, w1b, w2b, params, y);
}

// ---------------------------------------------------------------------------
// Inference on the 5th-generation tensor cores (tcgen05): one CTA per SM
// keeps W1 and W2 in shared memory; per tile of 128 rows one elected thread
// issues layer 1 (M=128, N=128, K=96 as 6 MMAs of K=16) into TMEM columns
// 0..127, the 4 warps read their 32 TMEM lanes (one row each), add b1,
// apply GELU, round to BF16 and store the row as layer 2's A operand; layer 2
// (K=128) goes to TMEM columns 128..255; the epilogue applies b2, GELU, BF16
// rounding and the FP32 layer 3.  Operands use the no-swizzle K-major
// layout: 8x8 core matrices (8 rows of 16 bytes) contiguous, LBO = 128 bytes
// between core matrices along K, SBO = (K/8)*128 bytes between 8-row groups.
// Every wait is bounded: on a timeout the CTA records err[0] and stops
// issuing, waits (bounded) for its MMAs in flight and frees its TMEM.
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);  // version 1, no swizzle
}
// kind::f16, BF16 A and B (K-major), FP32 D, M = 128, N = 128
constexpr uint32_t UMMA_IDESC = (1u << 4) | (1u << 7) | (1u << 10) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
__device__ __forceinline__ void umma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(UMMA_IDESC), "r"(acc));
}
__device__ __forceinline__ void umma_commit(uint64_t *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
               : "memory");
}
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t phase, long limit) {
  for (long it = 0; it < limit; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    if (ok) return true;
  }
  return false;
}
__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }
// 32 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float v[32]) {
  uint32_t r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,%16,%17,%18,"
      "%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
        "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
        "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
        "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 32; ++q) v[q] = __uint_as_float(r[q]);
}
// byte offset of element (row, k) in the no-swizzle K-major layout with K columns
__host__ __device__ constexpr uint32_t kmaj_off(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K / 8) * 128 + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}
constexpr int TC_M = 128;
// One CTA per SM holds W1, W2 and the split layer-3 weights once; its four
// warpgroups each run their own tile pipeline (X tile -> layer 1 -> GELU ->
// layer 2 -> GELU -> layer 3) in a private 32 KB operand region and 128 TMEM
// columns, so that one group's MMAs run while the others are in their
// epilogues.  The TMEM columns are reused layer after layer (each epilogue
// has read them completely before the next MMA is issued) and the operand
// region likewise (X, then H1, then H2: each is dead once the MMA that reads
// it has completed).  Layer 1 multiplies the BF16 features by BF16 W1; the
// GELU epilogues run in packed half precision and store 2 gelu(z) as F16, so
// layers 2 and 3 are F16 x F16 products with W2 / 2 and W3 / 2 (exact
// halvings).  Layer 3 (3 outputs) runs on the tensor cores as well, N = 16:
// B rows 0..2 hold f16(W3/2) and rows 3..5 the F16 remainder, so
// y = D[:, o] + D[:, 3 + o] carries W3 to about 22 significant bits with FP32
// accumulation, like the FP32 layer 3 it replaces.
constexpr int TC_GROUPS = 4, TC_THREADS = 128 * TC_GROUPS;
constexpr int TC_REGION = TC_M * NH * 2;   // bytes of one group's X / H1 / H2 region
constexpr int TC_W3ROWS = 16;
constexpr size_t TC_SMEM = (size_t)(NH * NIN + NH * NH + TC_W3ROWS * NH) * sizeof(bf16) +
                           (size_t)TC_GROUPS * TC_REGION + (size_t)(2 * NH + 4) * sizeof(float) + 128;
// kind::f16 with F16 A and B (K-major), FP32 D, M = 128: N = 128 (layer 2)
// and N = 16 (layer 3)
constexpr uint32_t UMMA_IDESC_H = (1u << 4) | ((128u >> 3) << 17) | ((128u >> 4) << 24);
constexpr uint32_t UMMA_IDESC_H_N16 = (1u << 4) | ((16u >> 3) << 17) | ((128u >> 4) << 24);
__device__ __forceinline__ void umma_f16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(acc));
}
// 8 consecutive FP32 columns of this thread's TMEM lane
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float v[8]) {
  uint32_t r[8];
  asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
               : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
               : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int q = 0; q < 8; ++q) v[q] = __uint_as_float(r[q]);
}
__device__ __forceinline__ void group_sync(int g) {
  asm volatile("bar.sync %0, %1;" ::"r"(1 + g), "r"(128) : "memory");
}
__device__ __forceinline__ void cp_async16(void *dst, const void *src, bool valid) {
  const uint32_t d = smem_u32(dst);
  const int n = valid ? 16 : 0;  // zero-fill rows beyond n
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(n));
}
__device__ __forceinline__ uint32_t h2_bits(__half2 h) { return *reinterpret_cast<uint32_t *>(&h); }
__device__ __forceinline__ __half2 bits_h2(uint32_t u) { return *reinterpret_cast<__half2 *>(&u); }
__device__ __forceinline__ __half2 tanh_h2(__half2 x) {
  uint32_t y;
  asm("tanh.approx.f16x2 %0, %1;" : "=r"(y) : "r"(h2_bits(x)));
  return bits_h2(y);
}
// Twice the GELU of 32 accumulator columns plus bias, x (1 + tanh(c x (1 +
// a x^2))) with x = z + b, in packed half precision (two columns per
// instruction), into the next layer's K-major F16 A operand (row r, columns
// col0..col0+31).  The factor 1/2 is carried by the next layer's weights.
// bias2: the layer's biases as F16 pairs.
__device__ __forceinline__ void gelu2_store32(const float v[32], const uint32_t *bias2, int col0, unsigned char *A,
                                              int r) {
  const __half2 c0 = __float2half2_rn(0.7978845608028654f), c1 = __float2half2_rn(0.7978845608028654f * 0.044715f);
#pragma unroll
  for (int c8 = 0; c8 < 32; c8 += 8) {
    const uint4 bq = *reinterpret_cast<const uint4 *>(bias2 + (col0 + c8) / 2);
    const uint32_t bb[4] = {bq.x, bq.y, bq.z, bq.w};
    uint32_t pk[4];
#pragma unroll
    for (int e = 0; e < 4; ++e) {
      const __half2 x = __hadd2(__floats2half2_rn(v[c8 + 2 * e], v[c8 + 2 * e + 1]), bits_h2(bb[e]));
      const __half2 in = __hmul2(x, __hfma2(c1, __hmul2(x, x), c0));
      pk[e] = h2_bits(__hfma2(x, tanh_h2(in), x));
    }
    *reinterpret_cast<uint4 *>(A + kmaj_off(r, col0 + c8, NH)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
  }
}

// The 96 features of point t (as k_ibm_features_f forms them: the 27 taps
// minus U, U - u~, U, the normal component, F0 dt and the centre weight of
// each velocity component, standardised and rounded to BF16) into row r of
// the K-major operand tile, with the first pass's point force
// F0 = (U - u~)/dt to fxl.  Taps are read from the fields directly (the
// 3-float rows of a stencil share cache lines with the tile's neighbouring
// points).  Rows beyond the points, or points not active (l >= nla), get
// zero features.
__device__ __forceinline__ void feature_row(const FeatIn &fi, long t, unsigned char *A, int r) {
  const long npl = (long)fi.np * fi.nl;
  const int p = t < npl ? (int)(t / fi.nl) : 0;
  if (t >= npl || (int)(t - (long)p * fi.nl) >= fi.nla[p]) {
#pragma unroll
    for (int c8 = 0; c8 < NIN; c8 += 8) *reinterpret_cast<uint4 *>(A + kmaj_off(r, c8, NIN)) = make_uint4(0, 0, 0, 0);
    return;
  }
  const Geo &g = fi.g;
  const int4 ref = fi.pref[p];
  const float4 cf = fi.pcen[p];
  const PointRec rr = fi.rec[t];
  // the normal's scale (FP32 constants of the launch: no FP64 conversions
  // per point, which this GPU issues on its 1/64-rate FP64 pipe)
  const float inv_r = fi.pradfp ? (float)(1. / fi.pradfp[p]) : fi.inv_r;
#pragma unroll 1
  for (int c = 0; c < 3; ++c) {
    const CompStencil s = make_cs(rr, c, ref.z, g.K);
    const float *F = fi.F[c];
    // the rigid-body velocity as an FP32 pair (per point with rotation)
    float2 Us;
    if (fi.rotation) {
      const double Ud = fi.U[c][t];
      Us.x = (float)Ud;
      Us.y = (float)(Ud - (double)Us.x);
    } else {
      const float4 vh = fi.pvh[p], vl = fi.pvl[p];
      Us = c == 0 ? make_float2(vh.x, vl.x) : (c == 1 ? make_float2(vh.y, vl.y) : make_float2(vh.z, vl.z));
    }
    const float Uc = Us.x;
    float f[FEAT_PER_COMP];
    float acc = 0.f;
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
      for (int j = 0; j < 3; ++j) {
        const float wyz = s.w[3 + j] * s.w[6 + k];
        const int y = wrapm(ref.y + s.b[1] + j, g.J);
#pragma unroll
        for (int i = 0; i < 3; ++i) {
          const float tv = __ldg(&F[fidx(g, wrapm(ref.x + s.b[0] + i, g.I), y, s.b[2] + k)]);
          acc += tv * (s.w[i] * wyz);
          f[(k * 3 + j) * 3 + i] = tv - Uc;
        }
      }
    const float F0 = ((Uc - acc) + Us.y) * fi.dtif;  // (U - u~)/dt, as the first plain pass forms it
    fi.Fl[c][t] = F0;
    f[27] = Uc - acc;
    f[28] = Uc;
    const int dc = c == 0 ? rec_dx(rr.rel) : (c == 1 ? rec_dy(rr.rel) : rec_dz(rr.rel));
    const float frc = c == 0 ? rr.fx : (c == 1 ? rr.fy : rr.fz);
    const float cfc = c == 0 ? cf.x : (c == 1 ? cf.y : cf.z);
    const float hc = c == 0 ? fi.hx : (c == 1 ? fi.hy : fi.hz);
    f[29] = rec_armf(dc, frc, cfc, hc) * inv_r;
    f[30] = F0 * fi.dtf;
    f[31] = s.w[3 * c + 1];
    const float *mu = fi.mu + FEAT_PER_COMP * c, *is = fi.isig + FEAT_PER_COMP * c;
#pragma unroll
    for (int q = 0; q < FEAT_PER_COMP; q += 8) {
      uint32_t pk[4];
#pragma unroll
      for (int e = 0; e < 4; ++e) {
        __nv_bfloat162 h = __floats2bfloat162_rn((f[q + 2 * e] - __ldg(&mu[q + 2 * e])) * __ldg(&is[q + 2 * e]),
                                                 (f[q + 2 * e + 1] - __ldg(&mu[q + 2 * e + 1])) * __ldg(&is[q + 2 * e + 1]));
        pk[e] = *reinterpret_cast<uint32_t *>(&h);
      }
      *reinterpret_cast<uint4 *>(A + kmaj_off(r, FEAT_PER_COMP * c + q, NIN)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
    }
  }
}

template <bool FUSED>
__global__ void __launch_bounds__(TC_THREADS, 1) k_mlp_infer_tc(const bf16 *__restrict__ x, int n,
                                                                const bf16 *__restrict__ w1b,
                                                                const float *__restrict__ params,
                                                                float *__restrict__ y, int *__restrict__ err,
                                                                const FeatIn fi) {
  extern __shared__ __align__(16) unsigned char tc_sm[];
  unsigned char *W1c = tc_sm;                                 // [128 x 96]  K-major
  unsigned char *W2c = W1c + NH * NIN * 2;                    // [128 x 128]
  unsigned char *W3c = W2c + NH * NH * 2;                     // [16 x 128]
  unsigned char *R0 = W3c + TC_W3ROWS * NH * 2;               // group regions
  float *cst = reinterpret_cast<float *>(R0 + TC_GROUPS * TC_REGION);  // b1, b2 (F16 pairs), b3
  uint32_t *hb = reinterpret_cast<uint32_t *>(cst);
  uint64_t *bars = reinterpret_cast<uint64_t *>(cst + 2 * NH + 4);     // one per group
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bars + TC_GROUPS);
  int *gbad = reinterpret_cast<int *>(tslot + 1);  // per group: an MMA wait timed out
  const int tid = threadIdx.x, warp = tid >> 5, g = warp >> 2, gt = tid & 127;
  // weights into the K-major layouts (16-byte chunks), constants
  for (int q = tid; q < NH * NIN / 8; q += blockDim.x) {
    const int r = q / (NIN / 8), c8 = (q % (NIN / 8)) * 8;
    *reinterpret_cast<uint4 *>(W1c + kmaj_off(r, c8, NIN)) = *reinterpret_cast<const uint4 *>(&w1b[r * NIN + c8]);
  }
  for (int q = tid; q < NH * NH / 2; q += blockDim.x) {  // W2 / 2 in F16 (the epilogues store 2 gelu)
    const int r = q / (NH / 2), k = (q % (NH / 2)) * 2;
    const float2 w = *reinterpret_cast<const float2 *>(&params[OFF_W2 + r * NH + k]);
    *reinterpret_cast<__half2 *>(W2c + kmaj_off(r, k, NH)) = __floats2half2_rn(0.5f * w.x, 0.5f * w.y);
  }
  for (int q = tid; q < TC_W3ROWS * NH; q += blockDim.x) {  // W3 / 2 split into hi and lo F16 rows
    const int r = q / NH, k = q % NH;
    __half v = __float2half_rn(0.f);
    if (r < 2 * NOUT) {
      const float w = 0.5f * params[OFF_W3 + (r % NOUT) * NH + k];
      const __half hi = __float2half_rn(w);
      v = r < NOUT ? hi : __float2half_rn(w - __half2float(hi));
    }
    *reinterpret_cast<__half *>(W3c + kmaj_off(r, k, NH)) = v;
  }
  for (int t = tid; t < NH / 2; t += blockDim.x) {
    hb[t] = h2_bits(__floats2half2_rn(params[OFF_B1 + 2 * t], params[OFF_B1 + 2 * t + 1]));
    hb[NH / 2 + t] = h2_bits(__floats2half2_rn(params[OFF_B2 + 2 * t], params[OFF_B2 + 2 * t + 1]));
  }
  if (tid < NOUT) cst[NH + tid] = params[OFF_B3 + tid];
  if (warp == 0) {  // 512 TMEM columns: 128 per group
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid < TC_GROUPS) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(&bars[tid])));
    gbad[tid] = 0;
  }
  if (tid == 0) asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t D = *tslot + (uint32_t)(g * 128);
  const uint32_t lane_base = (uint32_t)((warp & 3) * 32) << 16;  // warp w of the group reads lanes 32w..
  unsigned char *A = R0 + g * TC_REGION;
  uint64_t *bar = &bars[g];
  const uint32_t *hb1 = hb, *hb2 = hb + NH / 2;
  const float *b3 = cst + NH;
  const long LIMIT = 1L << 22;
  uint32_t phase = 0;
  const int ntiles = (n + TC_M - 1) / TC_M;
  const int r = gt;  // this thread's row of the tile (its TMEM lane)
  const uint32_t aa = smem_u32(A);
  // every thread of the group waits (bounded) for the group's MMAs; the
  // group then decides together whether to go on
  auto wait_mma = [&]() -> bool {
    if (!mbar_wait(bar, phase, LIMIT)) {
      if (err) atomicExch(err, 1);
      gbad[g] = 1;
    }
    phase ^= 1u;
    tc_fence_after();
    group_sync(g);
    return gbad[g] == 0;
  };
  for (int tile = blockIdx.x * TC_GROUPS + g; tile < ntiles; tile += gridDim.x * TC_GROUPS) {
    const long row0 = (long)tile * TC_M;
    if constexpr (FUSED) {
      feature_row(fi, row0 + gt, A, gt);  // this thread's row of the X tile
    } else {
      // X tile (zero rows beyond n) by asynchronous 16-byte copies
      for (int q = gt; q < TC_M * NIN / 8; q += 128) {
        const int rr = q / (NIN / 8), c8 = (q % (NIN / 8)) * 8;
        const bool valid = row0 + rr < n;
        cp_async16(A + kmaj_off(rr, c8, NIN), valid ? &x[(row0 + rr) * NIN + c8] : x, valid);
      }
      asm volatile("cp.async.wait_all;\n" ::: "memory");
    }
    fence_async_smem();
    group_sync(g);
    if (gt == 0) {  // layer 1
      tc_fence_after();
      const uint32_t wa = smem_u32(W1c);
#pragma unroll
      for (int kk = 0; kk < NIN / 16; ++kk)
        umma_bf16(D, umma_desc(aa + kk * 256, 128, (NIN / 8) * 128), umma_desc(wa + kk * 256, 128, (NIN / 8) * 128),
                  kk > 0);
      umma_commit(bar);
    }
    if (!wait_mma()) break;
    // epilogue 1: H1 = f16(2 gelu(D + b1)) over X (dead once layer 1 completed)
#pragma unroll 1
    for (int cc = 0; cc < 4; ++cc) {
      float v[32];
      tmem_ld32(D + lane_base + cc * 32, v);
      gelu2_store32(v, hb1, cc * 32, A, r);
    }
    tc_fence_before();
    fence_async_smem();
    group_sync(g);
    if (gt == 0) {  // layer 2 into the same columns (read completely above)
      tc_fence_after();
      const uint32_t wa = smem_u32(W2c);
#pragma unroll
      for (int kk = 0; kk < NH / 16; ++kk)
        umma_f16(D, umma_desc(aa + kk * 256, 128, (NH / 8) * 128), umma_desc(wa + kk * 256, 128, (NH / 8) * 128),
                 UMMA_IDESC_H, kk > 0);
      umma_commit(bar);
    }
    if (!wait_mma()) break;
    // epilogue 2: H2 = f16(2 gelu(D + b2)) over H1
#pragma unroll 1
    for (int cc = 0; cc < 4; ++cc) {
      float v[32];
      tmem_ld32(D + lane_base + cc * 32, v);
      gelu2_store32(v, hb2, cc * 32, A, r);
    }
    tc_fence_before();
    fence_async_smem();
    group_sync(g);
    if (gt == 0) {  // layer 3: N = 16 (W3 hi and lo rows)
      tc_fence_after();
      const uint32_t wa = smem_u32(W3c);
#pragma unroll
      for (int kk = 0; kk < NH / 16; ++kk)
        umma_f16(D, umma_desc(aa + kk * 256, 128, (NH / 8) * 128), umma_desc(wa + kk * 256, 128, (NH / 8) * 128),
                 UMMA_IDESC_H_N16, kk > 0);
      umma_commit(bar);
    }
    if (!wait_mma()) break;
    float v[8];
    tmem_ld8(D + lane_base, v);
    if (row0 + r < n)
      for (int o = 0; o < NOUT; ++o) y[(row0 + r) * NOUT + o] = (v[o] + v[NOUT + o]) + b3[o];
    tc_fence_before();
    group_sync(g);  // D and A are reused by the next tile
  }
  // a timed-out MMA may still be running: give it a bounded time to land
  // (the parity that timed out; wait_mma has already flipped `phase`)
  if (gbad[g] && gt == 0) mbar_wait(bar, phase ^ 1u, LIMIT);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(*tslot));
}
int launch_mlp_infer_tc(cudaStream_t s, const bf16 *x, int n, const bf16 *w1b, const bf16 *w2b, const float *params,
                        float *y, int *err) {
  (void)w2b;  // layers 2 and 3 take F16 copies of the FP32 weights in params
  if (n <= 0) return 0;
  const int ntiles = (n + TC_M - 1) / TC_M;
  const int nblk = (ntiles + TC_GROUPS - 1) / TC_GROUPS;
  const int grid = nblk < 152 ? nblk : 152;
  k_mlp_infer_tc<false><<<grid, TC_THREADS, TC_SMEM, s>>>(x, n, w1b, params, y, err, FeatIn{});
  return 1;
}
int launch_mlp_features_tc(cudaStream_t s, const FeatIn &fi, const bf16 *w1b, const float *params, float *y,
                           int *err) {
  const long n = (long)fi.np * fi.nl;
  if (n <= 0) return 0;
  const int ntiles = (int)((n + TC_M - 1) / TC_M);
  const int nblk = (ntiles + TC_GROUPS - 1) / TC_GROUPS;
  const int grid = nblk < 152 ? nblk : 152;
  k_mlp_infer_tc<true><<<grid, TC_THREADS, TC_SMEM, s>>>(nullptr, (int)n, w1b, params, y, err, fi);
  return 1;
}

// ---------------------------------------------------------------------------
// Training on the 5th-generation tensor cores (tcgen05): one CTA per 128-row
// tile of the batch runs the forward pass, the backward pass and the tile's
// weight gradients; a second kernel sums the tiles' gradients in a fixed
// order and applies Adam.  Rounding points as the CPU reference of the model
// states them: BF16 features, W1, W2, hidden activations and back-propagated
// pre-activation gradients; FP32 accumulation (TMEM); FP32 layer 3.
//
// Every operand is one shared-memory tile of 8x8 core matrices (8 rows of 16
// bytes, row groups `sbo` bytes apart, column groups 128 bytes apart), and
// the same tile serves as a K-major operand (rows = M or N) and, through a
// second descriptor, as an MN-major one (rows = K): the forward products
// read X, H1 and W1, W2 K-major; dH1 = dZ2 W2 reads W2 MN-major; the weight
// gradients, whose K is the tile's 128 rows, read dZ2, dZ1, H1, H2, X and dY
// MN-major.  A column of ones appended to X and to H1 turns the bias
// gradients of layers 1 and 2 into one more output column of dW1 and dW2.
// dY enters the layer-3 weight gradient as a BF16 pair (hi + lo), so that
// product keeps about 16 significant bits of dY.
//
// TMEM (512 columns): Z1 [0,128) -> dW1|db1 [0,112) once Z1 is dead;
// Z2 [128,256) -> dH1 [128,256); dW2|db2 [256,400); dW3^T (hi, lo) [400,416).
// Every wait is bounded: on a timeout the CTA records err[0] and stops
// issuing, waits (bounded) for its MMA in flight and frees its TMEM.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned mix32(unsigned x) {
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}
// byte offset of element (row, col) of a core-matrix tile with row groups
// sbo bytes apart
__host__ __device__ constexpr uint32_t cm_off(int row, int col, uint32_t sbo) {
  return (uint32_t)((row >> 3) * sbo + (col >> 3) * 128 + (row & 7) * 16 + (col & 7) * 2);
}
// kind::f16 instruction descriptor: BF16 A and B, FP32 D; amn / bmn: the
// operand is MN-major
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N, int amn, int bmn) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)amn << 15) | ((uint32_t)bmn << 16) |
         ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// MN-major no-swizzle descriptor: K groups (8 rows of the tile) kstride
// bytes apart (leading byte offset), MN groups 128 bytes apart (stride
// byte offset)
__device__ __forceinline__ uint64_t mn_desc(uint32_t saddr, uint32_t kstride) { return umma_desc(saddr, kstride, 128); }

constexpr int TT_THREADS = 256;
constexpr int TT_XK = NIN + 16;   // X, a column of ones, zeros
constexpr int TT_HK = NH + 16;    // H1, a column of ones, zeros
constexpr int TT_DYN = 16;        // dY hi (columns 0..2), lo (3..5), zeros
constexpr uint32_t TT_SB_X = TT_XK / 8 * 128, TT_SB_H1 = TT_HK / 8 * 128, TT_SB_H = NH / 8 * 128,
                   TT_SB_W1 = NIN / 8 * 128, TT_SB_DY = TT_DYN / 8 * 128;
constexpr size_t TT_OW1 = 0, TT_OW2 = TT_OW1 + NH * NIN * 2, TT_OX = TT_OW2 + NH * NH * 2,
                 TT_OH1 = TT_OX + 128 * TT_XK * 2, TT_OH2 = TT_OH1 + 128 * TT_HK * 2, TT_OD2 = TT_OH2 + 128 * NH * 2,
                 TT_ODY = TT_OD2 + 128 * NH * 2, TT_OF = TT_ODY + 128 * TT_DYN * 2;
// FP32 constants: b1, b2, W3, b3, the two column halves' layer-3 partials,
// per-warp sums of dY and the squared error
constexpr int TF_B1 = 0, TF_B2 = NH, TF_W3 = 2 * NH, TF_B3 = TF_W3 + NOUT * NH, TF_YP = TF_B3 + 4,
              TF_RED = TF_YP + 2 * 128 * 4, TF_N = TF_RED + 4 * 4;
// The CTA takes the whole 227 KB (it holds all 512 TMEM columns, one CTA per
// SM in any case): every descriptor's reach, with its two byte offsets read
// either way round, stays inside the allocation.
constexpr size_t TT_OBAR = TT_OF + TF_N * 4, TT_SMEM = 227 * 1024;
constexpr int TT_PSTRIDE = (NPARAM + 1 + 3) / 4 * 4;  // a tile's gradient, then its loss
static_assert(TT_OBAR % 8 == 0 && TT_OBAR + 32 <= TT_SMEM, "training kernel shared memory");
static_assert(TT_OD2 + 7 * 2 * TT_SB_H + 128 + 15 * TT_SB_H + 127 < TT_SMEM &&
                  TT_OH1 + 7 * 2 * TT_SB_H1 + 128 + 17 * TT_SB_H1 + 127 < TT_SMEM,
              "MN-major operand reach");
constexpr uint32_t ID_L1 = idesc_bf16(128, NH, 0, 0), ID_L2 = idesc_bf16(128, NH, 0, 0),
                   ID_DH1 = idesc_bf16(128, NH, 0, 1), ID_DW2 = idesc_bf16(128, TT_HK, 1, 1),
                   ID_DW3 = idesc_bf16(128, TT_DYN, 1, 1), ID_DW1 = idesc_bf16(128, TT_XK, 1, 1);

struct MlpTrainArgs {
  const bf16 *X;    // [n][96] standardised features
  const float *T;   // [n][3] standardised targets
  int n, nb, gather;
  unsigned seed;
  int step;
  const bf16 *w1b, *w2b;
  const float *params;
  float *part;      // [tiles][TT_PSTRIDE]
  float *y;         // outputs [nb][3] or null
  int *err;
};
// row `row` of the batch: drawn with replacement by a counter-based hash of
// (seed, step, row), or the row itself
__device__ __forceinline__ int train_src(const MlpTrainArgs &A, int row) {
  if (!A.gather) return row;
  const unsigned h = mix32(A.seed ^ mix32((unsigned)A.step * 0x9E3779B9U + (unsigned)row));
  return (int)(h % (unsigned)A.n);
}
__device__ __forceinline__ uint32_t bf2_bits(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t *>(&v);
}
__device__ __forceinline__ void st4f(float *p, const float *v) {
  *reinterpret_cast<float4 *>(p) = make_float4(v[0], v[1], v[2], v[3]);
}

__global__ void __launch_bounds__(TT_THREADS, 1) k_mlp_train_tc(const MlpTrainArgs A) {
  extern __shared__ __align__(16) unsigned char tt_sm[];
  unsigned char *W1s = tt_sm + TT_OW1, *W2s = tt_sm + TT_OW2, *Xs = tt_sm + TT_OX, *H1s = tt_sm + TT_OH1,
                *H2s = tt_sm + TT_OH2, *D2s = tt_sm + TT_OD2, *DYs = tt_sm + TT_ODY;
  float *fs = reinterpret_cast<float *>(tt_sm + TT_OF);
  uint64_t *bar = reinterpret_cast<uint64_t *>(tt_sm + TT_OBAR);
  uint32_t *tslot = reinterpret_cast<uint32_t *>(bar + 1);
  int *bad = reinterpret_cast<int *>(tslot + 1);
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int row0 = blockIdx.x * 128;
  // the tile's rows of X (16-byte asynchronous copies; zero rows beyond nb),
  // the ones column, W1 and W2 (BF16), the FP32 constants
  for (int q = tid; q < 128 * (NIN / 8); q += TT_THREADS) {
    const int r = q / (NIN / 8), c8 = (q % (NIN / 8)) * 8;
    const bool valid = row0 + r < A.nb;
    cp_async16(Xs + cm_off(r, c8, TT_SB_X), valid ? A.X + (long)train_src(A, row0 + r) * NIN + c8 : A.X, valid);
  }
  for (int q = tid; q < 128 * 2; q += TT_THREADS) {
    const int r = q >> 1, c8 = NIN + (q & 1) * 8;
    const uint32_t one = (c8 == NIN && row0 + r < A.nb) ? 0x3F80u : 0u;  // BF16 1.0 in column 96
    *reinterpret_cast<uint4 *>(Xs + cm_off(r, c8, TT_SB_X)) = make_uint4(one, 0u, 0u, 0u);
  }
  for (int q = tid; q < NH * NIN / 8; q += TT_THREADS) {
    const int r = q / (NIN / 8), c8 = (q % (NIN / 8)) * 8;
    cp_async16(W1s + cm_off(r, c8, TT_SB_W1), A.w1b + r * NIN + c8, true);
  }
  for (int q = tid; q < NH * NH / 8; q += TT_THREADS) {
    const int r = q / (NH / 8), c8 = (q % (NH / 8)) * 8;
    cp_async16(W2s + cm_off(r, c8, TT_SB_H), A.w2b + r * NH + c8, true);
  }
  for (int q = tid; q < NH; q += TT_THREADS) {
    fs[TF_B1 + q] = A.params[OFF_B1 + q];
    fs[TF_B2 + q] = A.params[OFF_B2 + q];
  }
  for (int q = tid; q < NOUT * NH; q += TT_THREADS) fs[TF_W3 + q] = A.params[OFF_W3 + q];
  if (tid < NOUT) fs[TF_B3 + tid] = A.params[OFF_B3 + tid];
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(tslot)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)));
    *bad = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t T0 = *tslot;
  const int q4 = warp & 3, hf = warp >> 2;  // TMEM lane quarter, column half
  const int r = q4 * 32 + lane;              // this thread's row of the tile (its TMEM lane)
  const uint32_t lb = (uint32_t)(q4 * 32) << 16;
  const bool valid = row0 + r < A.nb;
  const uint32_t xs = smem_u32(Xs), w1 = smem_u32(W1s), w2 = smem_u32(W2s), h1 = smem_u32(H1s), h2 = smem_u32(H2s),
                 d2 = smem_u32(D2s), dys = smem_u32(DYs);
  const long LIMIT = 1L << 22;
  uint32_t phase = 0;
  // all threads wait (bounded) for the committed MMAs, then decide together
  auto mma_wait = [&]() -> bool {
    if (!mbar_wait(bar, phase, LIMIT)) {
      if (A.err) atomicExch(A.err, 1);
      *bad = 1;
    }
    phase ^= 1u;
    tc_fence_after();
    __syncthreads();
    return *bad == 0;
  };
  auto issued = [&]() {  // operands written by the threads, visible to the tensor cores
    tc_fence_before();
    fence_async_smem();
    __syncthreads();
  };

  // ---- layer 1: Z1 = X W1^T -> TMEM [0,128)
  if (tid == 0) {
    tc_fence_after();
#pragma unroll
    for (int kk = 0; kk < NIN / 16; ++kk)
      umma_f16(T0, umma_desc(xs + kk * 256, 128, TT_SB_X), umma_desc(w1 + kk * 256, 128, TT_SB_W1), ID_L1, kk > 0);
    umma_commit(bar);
  }
  bool ok = mma_wait();
  // H1 = bf16(gelu(Z1 + b1)), and the ones column
  if (ok) {
#pragma unroll 1
    for (int cc = 0; cc < 2; ++cc) {
      const int col = hf * 64 + cc * 32;
      float v[32];
      tmem_ld32(T0 + lb + col, v);
#pragma unroll
      for (int c8 = 0; c8 < 32; c8 += 8) {
        uint32_t pk[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int c = col + c8 + 2 * e;
          pk[e] = bf2_bits(gelu_f(v[c8 + 2 * e] + fs[TF_B1 + c]), gelu_f(v[c8 + 2 * e + 1] + fs[TF_B1 + c + 1]));
        }
        *reinterpret_cast<uint4 *>(H1s + cm_off(r, col + c8, TT_SB_H1)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
    if (hf == 1) {
      *reinterpret_cast<uint4 *>(H1s + cm_off(r, NH, TT_SB_H1)) = make_uint4(valid ? 0x3F80u : 0u, 0u, 0u, 0u);
      *reinterpret_cast<uint4 *>(H1s + cm_off(r, NH + 8, TT_SB_H1)) = make_uint4(0u, 0u, 0u, 0u);
    }
  }
  issued();
  // ---- layer 2: Z2 = H1 W2^T -> TMEM [128,256)
  if (ok && tid == 0) {
    tc_fence_after();
#pragma unroll
    for (int kk = 0; kk < NH / 16; ++kk)
      umma_f16(T0 + 128, umma_desc(h1 + kk * 256, 128, TT_SB_H1), umma_desc(w2 + kk * 256, 128, TT_SB_H), ID_L2,
               kk > 0);
    umma_commit(bar);
  }
  if (ok) ok = mma_wait();
  // H2 = bf16(gelu(Z2 + b2)); layer 3 on the FP32 pipes (each column half
  // a partial dot product)
  if (ok) {
    float yp[NOUT] = {0.f, 0.f, 0.f};
#pragma unroll 1
    for (int cc = 0; cc < 2; ++cc) {
      const int col = hf * 64 + cc * 32;
      float v[32];
      tmem_ld32(T0 + 128 + lb + col, v);
#pragma unroll
      for (int c8 = 0; c8 < 32; c8 += 8) {
        uint32_t pk[4];
#pragma unroll
        for (int e = 0; e < 4; ++e) {
          const int c = col + c8 + 2 * e;
          const __nv_bfloat162 hb =
              __floats2bfloat162_rn(gelu_f(v[c8 + 2 * e] + fs[TF_B2 + c]), gelu_f(v[c8 + 2 * e + 1] + fs[TF_B2 + c + 1]));
          const float ha = __low2float(hb), hc = __high2float(hb);
#pragma unroll
          for (int o = 0; o < NOUT; ++o) yp[o] += ha * fs[TF_W3 + o * NH + c] + hc * fs[TF_W3 + o * NH + c + 1];
          pk[e] = *reinterpret_cast<const uint32_t *>(&hb);
        }
        *reinterpret_cast<uint4 *>(H2s + cm_off(r, col + c8, TT_SB_H)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
#pragma unroll
    for (int o = 0; o < NOUT; ++o) fs[TF_YP + (hf * 128 + r) * 4 + o] = yp[o];
  }
  __syncthreads();
  if (ok) {
    // Y, dY = 2 (Y - T) / nb (zero beyond nb), the loss
    float dy[NOUT], e[NOUT];
    const long src = valid ? train_src(A, row0 + r) : 0;
#pragma unroll
    for (int o = 0; o < NOUT; ++o) {
      const float yv = (fs[TF_YP + r * 4 + o] + fs[TF_YP + (128 + r) * 4 + o]) + fs[TF_B3 + o];
      e[o] = valid ? yv - A.T[src * NOUT + o] : 0.f;
      dy[o] = (2.f / (float)A.nb) * e[o];
      if (hf == 0 && valid && A.y) A.y[(long)(row0 + r) * NOUT + o] = yv;
    }
    if (hf == 0) {
      float hi[NOUT], lo[NOUT];
#pragma unroll
      for (int o = 0; o < NOUT; ++o) {
        hi[o] = __bfloat162float(__float2bfloat16(dy[o]));
        lo[o] = dy[o] - hi[o];
      }
      *reinterpret_cast<uint4 *>(DYs + cm_off(r, 0, TT_SB_DY)) =
          make_uint4(bf2_bits(hi[0], hi[1]), bf2_bits(hi[2], lo[0]), bf2_bits(lo[1], lo[2]), 0u);
      *reinterpret_cast<uint4 *>(DYs + cm_off(r, 8, TT_SB_DY)) = make_uint4(0u, 0u, 0u, 0u);
      float s[4] = {dy[0], dy[1], dy[2], (e[0] * e[0] + e[1] * e[1] + e[2] * e[2]) / (float)A.nb};
#pragma unroll
      for (int k = 0; k < 4; ++k)
        for (int d = 16; d > 0; d >>= 1) s[k] += __shfl_xor_sync(0xffffffffu, s[k], d);
      if (lane == 0)
#pragma unroll
        for (int k = 0; k < 4; ++k) fs[TF_RED + q4 * 4 + k] = s[k];
    }
    // dZ2 = bf16((dY W3) gelu'(Z2 + b2)), Z2 read again
#pragma unroll 1
    for (int cc = 0; cc < 2; ++cc) {
      const int col = hf * 64 + cc * 32;
      float v[32];
      tmem_ld32(T0 + 128 + lb + col, v);
#pragma unroll
      for (int c8 = 0; c8 < 32; c8 += 8) {
        uint32_t pk[4];
#pragma unroll
        for (int ee = 0; ee < 4; ++ee) {
          float d[2];
#pragma unroll
          for (int u = 0; u < 2; ++u) {
            const int c = col + c8 + 2 * ee + u;
            const float dh = dy[0] * fs[TF_W3 + c] + dy[1] * fs[TF_W3 + NH + c] + dy[2] * fs[TF_W3 + 2 * NH + c];
            d[u] = dh * gelu_grad_f(v[c8 + 2 * ee + u] + fs[TF_B2 + c]);
          }
          pk[ee] = bf2_bits(d[0], d[1]);
        }
        *reinterpret_cast<uint4 *>(D2s + cm_off(r, col + c8, TT_SB_H)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
  }
  issued();
  // ---- dH1 = dZ2 W2 -> [128,256); [dW2 | db2] = dZ2^T [H1 | 1] -> [256,400);
  //      dW3^T (hi, lo) = H2^T [dY hi | dY lo] -> [400,416)
  if (ok && tid == 0) {
    tc_fence_after();
#pragma unroll
    for (int kk = 0; kk < NH / 16; ++kk)
      umma_f16(T0 + 128, umma_desc(d2 + kk * 256, 128, TT_SB_H), mn_desc(w2 + kk * 2 * TT_SB_H, TT_SB_H), ID_DH1,
               kk > 0);
#pragma unroll
    for (int kk = 0; kk < 128 / 16; ++kk)
      umma_f16(T0 + 256, mn_desc(d2 + kk * 2 * TT_SB_H, TT_SB_H), mn_desc(h1 + kk * 2 * TT_SB_H1, TT_SB_H1), ID_DW2,
               kk > 0);
#pragma unroll
    for (int kk = 0; kk < 128 / 16; ++kk)
      umma_f16(T0 + 400, mn_desc(h2 + kk * 2 * TT_SB_H, TT_SB_H), mn_desc(dys + kk * 2 * TT_SB_DY, TT_SB_DY), ID_DW3,
               kk > 0);
    umma_commit(bar);
  }
  if (ok) ok = mma_wait();
  // dZ1 = bf16(dH1 gelu'(Z1 + b1)) into H2's tile (read by the completed MMAs)
  if (ok) {
#pragma unroll 1
    for (int cc = 0; cc < 2; ++cc) {
      const int col = hf * 64 + cc * 32;
      float dh[32], z[32];
      tmem_ld32(T0 + 128 + lb + col, dh);
      tmem_ld32(T0 + lb + col, z);
#pragma unroll
      for (int c8 = 0; c8 < 32; c8 += 8) {
        uint32_t pk[4];
#pragma unroll
        for (int ee = 0; ee < 4; ++ee) {
          const int c = col + c8 + 2 * ee, j = c8 + 2 * ee;
          pk[ee] = bf2_bits(dh[j] * gelu_grad_f(z[j] + fs[TF_B1 + c]), dh[j + 1] * gelu_grad_f(z[j + 1] + fs[TF_B1 + c + 1]));
        }
        *reinterpret_cast<uint4 *>(H2s + cm_off(r, col + c8, TT_SB_H)) = make_uint4(pk[0], pk[1], pk[2], pk[3]);
      }
    }
  }
  issued();
  // ---- [dW1 | db1] = dZ1^T [X | 1] -> [0,112)
  if (ok && tid == 0) {
    tc_fence_after();
#pragma unroll
    for (int kk = 0; kk < 128 / 16; ++kk)
      umma_f16(T0, mn_desc(h2 + kk * 2 * TT_SB_H, TT_SB_H), mn_desc(xs + kk * 2 * TT_SB_X, TT_SB_X), ID_DW1, kk > 0);
    umma_commit(bar);
  }
  if (ok) ok = mma_wait();
  // the tile's gradient (TMEM lane = output neuron) and loss
  if (ok) {
    float *P = A.part + (long)blockIdx.x * TT_PSTRIDE;
    const int o = r;
    float v[32];
    if (hf == 0) {
#pragma unroll 1
      for (int cc = 0; cc < 2; ++cc) {
        tmem_ld32(T0 + lb + cc * 32, v);
#pragma unroll
        for (int k = 0; k < 32; k += 4) st4f(P + o * NIN + cc * 32 + k, v + k);
      }
    } else {
      tmem_ld32(T0 + lb + 64, v);
#pragma unroll
      for (int k = 0; k < 32; k += 4) st4f(P + o * NIN + 64 + k, v + k);
      float v8[8];
      tmem_ld8(T0 + lb + NIN, v8);
      P[OFF_B1 + o] = v8[0];
    }
#pragma unroll 1
    for (int cc = 0; cc < 2; ++cc) {
      const int col = hf * 64 + cc * 32;
      tmem_ld32(T0 + 256 + lb + col, v);
#pragma unroll
      for (int k = 0; k < 32; k += 4) st4f(P + OFF_W2 + o * NH + col + k, v + k);
    }
    float v8[8];
    if (hf == 1) {
      tmem_ld8(T0 + 256 + NH + lb, v8);
      P[OFF_B2 + o] = v8[0];
    } else {
      tmem_ld8(T0 + 400 + lb, v8);
#pragma unroll
      for (int k = 0; k < NOUT; ++k) P[OFF_W3 + k * NH + o] = v8[k] + v8[NOUT + k];
    }
    if (tid == 0)
#pragma unroll
      for (int k = 0; k < 4; ++k) {
        const float s = ((fs[TF_RED + k] + fs[TF_RED + 4 + k]) + fs[TF_RED + 8 + k]) + fs[TF_RED + 12 + k];
        if (k < NOUT) P[OFF_B3 + k] = s;
        else P[NPARAM] = s;
      }
  }
  // a timed-out MMA may still be running: give it a bounded time to land
  if (*bad && tid == 0) mbar_wait(bar, phase ^ 1u, LIMIT);
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(T0));
}

// the tiles' gradients summed in tile order (deterministic) into grad and
// the loss; with adam: one Adam step of the FP32 masters and their BF16
// copies
__global__ void __launch_bounds__(256) k_mlp_reduce_adam(const float *__restrict__ part, int nparts,
                                                         float *__restrict__ grad, float *__restrict__ loss,
                                                         float *__restrict__ p, float *__restrict__ m,
                                                         float *__restrict__ v, bf16 *__restrict__ w1b,
                                                         bf16 *__restrict__ w2b, int adam, float lr, float b1, float b2,
                                                         float eps, float c1, float c2) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t > NPARAM) return;
  float s = 0.f;
#pragma unroll 8
  for (int c = 0; c < nparts; ++c) s += part[(long)c * TT_PSTRIDE + t];
  if (t == NPARAM) {
    *loss = s;
    return;
  }
  grad[t] = s;
  if (!adam) return;
  const float mm = b1 * m[t] + (1.f - b1) * s;
  const float vv = b2 * v[t] + (1.f - b2) * s * s;
  m[t] = mm;
  v[t] = vv;
  const float pn = p[t] - lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  p[t] = pn;
  if (t < NH * NIN) w1b[t] = __float2bfloat16(pn);
  else if (t >= OFF_W2 && t < OFF_W2 + NH * NH) w2b[t - OFF_W2] = __float2bfloat16(pn);
}
__global__ void k_refresh_bf16(const float *__restrict__ p, bf16 *__restrict__ w1b, bf16 *__restrict__ w2b) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < NH * NIN + NH * NH; t += gridDim.x * blockDim.x) {
    if (t < NH * NIN) w1b[t] = __float2bfloat16(p[t]);
    else w2b[t - NH * NIN] = __float2bfloat16(p[OFF_W2 + t - NH * NIN]);
  }
}

int mlp_nparam() { return NPARAM; }
size_t mlp_part_floats(int nb) { return (size_t)((nb + 127) / 128) * TT_PSTRIDE; }

void launch_mlp_refresh(cudaStream_t s, const float *params, bf16 *w1b, bf16 *w2b) {
  k_refresh_bf16<<<64, 256, 0, s>>>(params, w1b, w2b);
}

// one optimisation step (adam = 1) or the gradient alone: rows drawn from
// X, T (n rows) by the (seed, step, row) hash (gather = 1), or rows 0..nb-1
int launch_mlp_train_step(cudaStream_t s, const MlpTrainBuffers &B, const bf16 *X, const float *T, int n, int nb,
                          unsigned seed, int gather, int step, float lr, int adam, float *y) {
  const int ntile = (nb + 127) / 128;
  const MlpTrainArgs A{X, T, n, nb, gather, seed, step, B.w1b, B.w2b, B.params, B.part, y, B.err};
  k_mlp_train_tc<<<ntile, TT_THREADS, TT_SMEM, s>>>(A);
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = adam ? 1.f - powf(b1, (float)step) : 1.f, c2 = adam ? 1.f - powf(b2, (float)step) : 1.f;
  k_mlp_reduce_adam<<<(NPARAM + 1 + 255) / 256, 256, 0, s>>>(B.part, ntile, B.grad, B.loss, B.params, B.m, B.v, B.w1b,
                                                             B.w2b, adam, lr, b1, b2, 1e-8f, c1, c2);
  return 2;
}

// harvested samples -> standardised training set: X (bf16), T (fp32)
__global__ void k_mlp_stage(int n, const float *__restrict__ feat, const float *__restrict__ targ,
                            const float *__restrict__ mu, const float *__restrict__ isig,
                            const float *__restrict__ tmu, const float *__restrict__ tsig, bf16 *__restrict__ X,
                            float *__restrict__ T) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < (long)n * NIN; q += (long)gridDim.x * blockDim.x) {
    const int c = (int)(q % NIN);
    X[q] = __float2bfloat16((feat[q] - mu[c]) * isig[c]);
  }
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < (long)n * NOUT; q += (long)gridDim.x * blockDim.x) {
    const int c = (int)(q % NOUT);
    T[q] = (targ[q] - tmu[c]) / tsig[c];
  }
}
void launch_mlp_stage(cudaStream_t s, int n, const float *feat, const float *targ, const float *mu, const float *isig,
                      const float *tmu, const float *tsig, bf16 *X, float *T) {
  k_mlp_stage<<<1216, 256, 0, s>>>(n, feat, targ, mu, isig, tmu, tsig, X, T);
}

// Standardisation of the harvested set: per column (96 features, 3
// targets) the mean and the standard deviation, two passes in FP64 over
// fixed row chunks (sums of the chunks in chunk order: deterministic).
// norm: mu[96], 1/sd[96] (0 for a constant column), target mu[3], sd[3]
// (1 for a constant column).
constexpr int NORM_BLOCKS = 608, NORM_COLS = NIN + NOUT;
__global__ void __launch_bounds__(128) k_mlp_colsum(int n, const float *__restrict__ feat,
                                                    const float *__restrict__ targ, const double *__restrict__ mu,
                                                    double *__restrict__ part) {
  const int c = threadIdx.x;
  if (c >= NORM_COLS) return;
  const long chunk = ((long)n + gridDim.x - 1) / gridDim.x;
  const long r0 = blockIdx.x * chunk, r1 = min((long)n, r0 + chunk);
  const double m = mu ? mu[c] : 0.;
  double s = 0.;
  for (long r = r0; r < r1; ++r) {
    const double a = c < NIN ? (double)feat[r * NIN + c] : (double)targ[r * NOUT + (c - NIN)];
    s += mu ? (a - m) * (a - m) : a;
  }
  part[(long)blockIdx.x * NORM_COLS + c] = s;
}
__global__ void k_mlp_colfinal(int n, int nblk, const double *__restrict__ part, double *__restrict__ mu,
                               float *__restrict__ norm, int second) {
  const int c = threadIdx.x;
  if (c >= NORM_COLS) return;
  double s = 0.;
  for (int b = 0; b < nblk; ++b) s += part[(long)b * NORM_COLS + c];
  s /= (double)n;
  if (!second) {
    mu[c] = s;
    if (c < NIN) norm[c] = (float)s;
    else norm[2 * NIN + (c - NIN)] = (float)s;
    return;
  }
  const double sd = sqrt(s);
  if (c < NIN) norm[NIN + c] = sd > 1e-30 ? (float)(1. / sd) : 0.f;
  else norm[2 * NIN + NOUT + (c - NIN)] = sd > 1e-30 ? (float)sd : 1.f;
}
size_t mlp_norm_scratch() { return (size_t)NORM_BLOCKS * NORM_COLS + NORM_COLS; }
int launch_mlp_norm(cudaStream_t s, int n, const float *feat, const float *targ, double *scratch, float *norm) {
  double *mu = scratch + (size_t)NORM_BLOCKS * NORM_COLS;
  k_mlp_colsum<<<NORM_BLOCKS, 128, 0, s>>>(n, feat, targ, nullptr, scratch);
  k_mlp_colfinal<<<1, 128, 0, s>>>(n, NORM_BLOCKS, scratch, mu, norm, 0);
  k_mlp_colsum<<<NORM_BLOCKS, 128, 0, s>>>(n, feat, targ, mu, scratch);
  k_mlp_colfinal<<<1, 128, 0, s>>>(n, NORM_BLOCKS, scratch, mu, norm, 1);
  return 4;
}

__global__ void k_f2bf(long n, const float *__restrict__ a, bf16 *__restrict__ b) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
    b[q] = __float2bfloat16(a[q]);
}
void launch_f2bf(cudaStream_t s, long n, const float *a, bf16 *b) { k_f2bf<<<608, 256, 0, s>>>(n, a, b); }

int mlp_set_smem_limits() {
  cudaError_t e = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_infer_smem());
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_infer_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_infer_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
  if (e == cudaSuccess)
    e = cudaFuncSetAttribute(k_mlp_train_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TT_SMEM);
  return e == cudaSuccess ? 0 : -1;
}

}  // namespace ibmk
