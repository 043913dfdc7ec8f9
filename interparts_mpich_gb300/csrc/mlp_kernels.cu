// mlp_kernels.cu -- learned multidirect-forcing correction.
//
// A per-Lagrangian-point MLP 96 -> 128 -> 128 -> 3 (tanh-form GELU) predicts
// the rest of the multidirect forcing after the first pass: from the slip
// left by pass 0 and the local velocity field it returns dF*dt, the
// velocity-unit correction that the plain passes 1 and 2 would add
// (interp_spread.f90 / forcing.f90, Nl = 3).
//
// Layers 1 and 2 run on the tensor cores: mma.sync m16n8k16 with BF16
// operands (features, weights, hidden activations) and FP32 accumulators;
// layer 3 (128 -> 3) and GELU run on the FP32 pipes.  Training (forward,
// backward, weight gradients, Adam) uses the same fragments; the FP32 master
// weights live on the device and BF16 copies are refreshed after each step.
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
constexpr int TILE = 64;                    // rows per CTA tile (4 warps x 16)
constexpr int OFF_B1 = NH * NIN, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH, OFF_W3 = OFF_B2 + NH,
              OFF_B3 = OFF_W3 + NOUT * NH, NPARAM = OFF_B3 + NOUT;

// ---------------------------------------------------------------------------
// Forward: X (N x 96, bf16) -> Y (N x 3, fp32).  Persistent CTAs keep W1, W2
// in shared memory.  TRAIN additionally stores Z1, Z2 (fp32) and H1, H2
// (bf16) for the backward pass.
// ---------------------------------------------------------------------------
struct MlpFwdArgs {
  const bf16 *x;
  int n;
  const bf16 *w1b, *w2b;
  const float *params;
  float *y;
  float *z1, *z2;
  bf16 *h1, *h2;
};

template <bool TRAIN>
__global__ void __launch_bounds__(128) k_mlp_forward(MlpFwdArgs A) {
  extern __shared__ __align__(16) unsigned char sm[];
  bf16 *W1s = reinterpret_cast<bf16 *>(sm);   // [128][LDX]
  bf16 *W2s = W1s + NH * LDX;                 // [128][LDH]
  bf16 *Xs = W2s + NH * LDH;                  // [64][LDX]
  bf16 *H1s = Xs + TILE * LDX;                // [64][LDH]
  bf16 *H2s = H1s + TILE * LDH;               // [64][LDH]
  float *bias = reinterpret_cast<float *>(H2s + TILE * LDH);  // b1, b2, W3, b3
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int t = tid; t < NH * NIN; t += blockDim.x) W1s[(t / NIN) * LDX + t % NIN] = A.w1b[t];
  for (int t = tid; t < NH * NH; t += blockDim.x) W2s[(t / NH) * LDH + t % NH] = A.w2b[t];
  for (int t = tid; t < NH; t += blockDim.x) { bias[t] = A.params[OFF_B1 + t]; bias[NH + t] = A.params[OFF_B2 + t]; }
  for (int t = tid; t < NOUT * NH + NOUT; t += blockDim.x) bias[2 * NH + t] = A.params[OFF_W3 + t];
  __syncthreads();
  const float *b1 = bias, *b2 = bias + NH, *w3 = bias + 2 * NH, *b3 = w3 + NOUT * NH;
  const int ntiles = (A.n + TILE - 1) / TILE;
  const int g = lane >> 2, tq = lane & 3;
  for (int tile = blockIdx.x; tile < ntiles; tile += gridDim.x) {
    const int row0 = tile * TILE;
    // stage the feature tile (rows beyond n are zero)
    for (int t = tid; t < TILE * NIN / 8; t += blockDim.x) {
      const int r = t / (NIN / 8), c8 = (t % (NIN / 8)) * 8;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (row0 + r < A.n) v = *reinterpret_cast<const uint4 *>(&A.x[(long)(row0 + r) * NIN + c8]);
      *reinterpret_cast<uint4 *>(&Xs[r * LDX + c8]) = v;
    }
    __syncthreads();
    const int m0 = warp * 16;
    // layer 1: 16 rows x 128 columns per warp
    float acc[16][4];
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < NIN; k0 += 16) {
      uint32_t a[4];
      load_a(a, Xs, LDX, m0, k0, lane);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        uint32_t b[2];
        load_b(b, W1s, LDX, j * 8, k0, lane);
        mma16816(acc[j], a, b);
      }
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int col = j * 8 + 2 * tq;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = m0 + g + 8 * h;
        const float z0 = acc[j][2 * h] + b1[col], z1 = acc[j][2 * h + 1] + b1[col + 1];
        const bf16 h0 = __float2bfloat16(gelu_f(z0)), h1v = __float2bfloat16(gelu_f(z1));
        H1s[r * LDH + col] = h0;
        H1s[r * LDH + col + 1] = h1v;
        if (TRAIN && row0 + r < A.n) {
          const long o = (long)(row0 + r) * NH + col;
          A.z1[o] = z0; A.z1[o + 1] = z1;
          A.h1[o] = h0; A.h1[o + 1] = h1v;
        }
      }
    }
    __syncwarp();
    // layer 2 (each warp reads only its own 16 rows of H1)
#pragma unroll
    for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
    for (int k0 = 0; k0 < NH; k0 += 16) {
      uint32_t a[4];
      load_a(a, H1s, LDH, m0, k0, lane);
#pragma unroll
      for (int j = 0; j < 16; ++j) {
        uint32_t b[2];
        load_b(b, W2s, LDH, j * 8, k0, lane);
        mma16816(acc[j], a, b);
      }
    }
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      const int col = j * 8 + 2 * tq;
#pragma unroll
      for (int h = 0; h < 2; ++h) {
        const int r = m0 + g + 8 * h;
        const float z0 = acc[j][2 * h] + b2[col], z1 = acc[j][2 * h + 1] + b2[col + 1];
        const bf16 h0 = __float2bfloat16(gelu_f(z0)), h1v = __float2bfloat16(gelu_f(z1));
        H2s[r * LDH + col] = h0;
        H2s[r * LDH + col + 1] = h1v;
        if (TRAIN && row0 + r < A.n) {
          const long o = (long)(row0 + r) * NH + col;
          A.z2[o] = z0; A.z2[o + 1] = z1;
          A.h2[o] = h0; A.h2[o + 1] = h1v;
        }
      }
    }
    __syncwarp();
    // layer 3 on the FP32 pipes: 16 rows x 3 outputs per warp
    for (int q = lane; q < 16 * NOUT; q += 32) {
      const int r = m0 + q / NOUT, o = q % NOUT;
      float s = b3[o];
      for (int c = 0; c < NH; ++c) s += __bfloat162float(H2s[r * LDH + c]) * w3[o * NH + c];
      if (row0 + r < A.n) A.y[(long)(row0 + r) * NOUT + o] = s;
    }
    __syncthreads();
  }
}

size_t mlp_forward_smem() {
  return (size_t)(NH * LDX + NH * LDH + TILE * LDX + 2 * TILE * LDH) * sizeof(bf16) +
         (size_t)(2 * NH + NOUT * NH + NOUT) * sizeof(float);
}

void launch_mlp_forward(cudaStream_t s, const bf16 *x, int n, const bf16 *w1b, const bf16 *w2b, const float *params,
                        float *y, float *z1, float *z2, bf16 *h1, bf16 *h2, int train) {
  if (n <= 0) return;
  MlpFwdArgs A{x, n, w1b, w2b, params, y, z1, z2, h1, h2};
  const int ntiles = (n + TILE - 1) / TILE;
  const int grid = ntiles < 2 * 152 ? ntiles : 2 * 152;
  if (train) k_mlp_forward<true><<<grid, 128, mlp_forward_smem(), s>>>(A);
  else k_mlp_forward<false><<<grid, 128, mlp_forward_smem(), s>>>(A);
}

// ---------------------------------------------------------------------------
// Inference: X (N x 96, bf16) -> Y (N x 3, fp32), one warp per 16-row tile.
// The layer-1 accumulators become the A fragments of layer 2 in registers:
// the m16n8k16 C fragment of the 8-column tiles 2m and 2m+1 holds exactly the
// A fragment of the 16-column k-block m (rows g, g+8; columns 2t, 2t+1 and
// 2t+8, 2t+9).  Layer 3 is a per-lane partial dot product over the 32
// columns a lane holds, summed over the 4 lanes of a row pair by shuffles.
// Same rounding points as the training forward: BF16 inputs, weights of
// layers 1-2 and hidden activations; FP32 accumulation; FP32 W3.
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
    const float F0 = ((Uc - acc) + Us.y) * (float)fi.dti;  // (U - u~)/dt, as the first plain pass forms it
    fi.Fl[c][t] = F0;
    f[27] = Uc - acc;
    f[28] = Uc;
    const int dc = c == 0 ? rec_dx(rr.rel) : (c == 1 ? rec_dy(rr.rel) : rec_dz(rr.rel));
    const float frc = c == 0 ? rr.fx : (c == 1 ? rr.fy : rr.fz);
    const float cfc = c == 0 ? cf.x : (c == 1 ? cf.y : cf.z);
    const float hc = (float)(c == 0 ? g.dx : (c == 1 ? g.dy : g.dz));
    f[29] = rec_armf(dc, frc, cfc, hc) * (fi.pradfp ? (float)(1. / fi.pradfp[p]) : fi.inv_r);
    f[30] = (float)F0 * (float)fi.dt;
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
// Backward through layer 3, GELU and layer 2 for a batch: dY = 2(Y-T)/B;
// dH2 = dY W3; dZ2 = dH2 * gelu'(Z2) (bf16); dH1 = dZ2 W2 (tensor cores);
// dZ1 = dH1 * gelu'(Z1) (bf16).  Bias and W3 gradients accumulate into grad.
// ---------------------------------------------------------------------------
struct MlpBwdArgs {
  int nb;
  const float *y, *t, *z1, *z2;
  const bf16 *h2;
  const bf16 *w2tb;  // W2 transposed: [in][out]
  const float *params;
  bf16 *dz1, *dz2;
  float *grad;
  float *loss;
};

__global__ void __launch_bounds__(128) k_mlp_backward(MlpBwdArgs A) {
  extern __shared__ __align__(16) unsigned char sm[];
  bf16 *W2t = reinterpret_cast<bf16 *>(sm);  // [128][LDH]: W2t[i][o]
  bf16 *D2 = W2t + NH * LDH;                 // [64][LDH] dZ2 tile
  float *w3 = reinterpret_cast<float *>(D2 + TILE * LDH);  // [3][128]
  float *dy = w3 + NOUT * NH;                              // [64][3]
  float *red = dy + TILE * NOUT;                           // [128] bias-gradient partials
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int t = tid; t < NH * NH; t += blockDim.x) W2t[(t / NH) * LDH + t % NH] = A.w2tb[t];
  for (int t = tid; t < NOUT * NH; t += blockDim.x) w3[t] = A.params[OFF_W3 + t];
  const int row0 = blockIdx.x * TILE;
  const float inv = 2.f / (float)A.nb;
  float lsum = 0.f;
  for (int q = tid; q < TILE * NOUT; q += blockDim.x) {
    const int r = q / NOUT, o = q % NOUT;
    float d = 0.f;
    if (row0 + r < A.nb) {
      const float e = A.y[(long)(row0 + r) * NOUT + o] - A.t[(long)(row0 + r) * NOUT + o];
      d = inv * e;
      lsum += e * e;
    }
    dy[q] = d;
  }
  __syncthreads();
  // loss, W3 and b3 gradients
  for (int q = tid; q < NOUT * NH + NOUT; q += blockDim.x) {
    float s = 0.f;
    if (q < NOUT * NH) {
      const int o = q / NH, c = q % NH;
      for (int r = 0; r < TILE && row0 + r < A.nb; ++r)
        s += dy[r * NOUT + o] * __bfloat162float(A.h2[(long)(row0 + r) * NH + c]);
      atomicAdd(&A.grad[OFF_W3 + q], s);
    } else {
      const int o = q - NOUT * NH;
      for (int r = 0; r < TILE; ++r) s += dy[r * NOUT + o];
      atomicAdd(&A.grad[OFF_B3 + o], s);
    }
  }
  for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
  if (lane == 0) atomicAdd(A.loss, lsum / (float)A.nb);
  // dZ2 = (dY W3) * gelu'(Z2)
  for (int q = tid; q < TILE * NH; q += blockDim.x) {
    const int r = q / NH, c = q % NH;
    float v = 0.f;
    if (row0 + r < A.nb) {
      const float dh = dy[r * NOUT] * w3[c] + dy[r * NOUT + 1] * w3[NH + c] + dy[r * NOUT + 2] * w3[2 * NH + c];
      v = dh * gelu_grad_f(A.z2[(long)(row0 + r) * NH + c]);
    }
    const bf16 vb = __float2bfloat16(v);
    D2[r * LDH + c] = vb;
    if (row0 + r < A.nb) A.dz2[(long)(row0 + r) * NH + c] = vb;
  }
  __syncthreads();
  // b2 gradient (sum of the rounded dZ2 over the tile rows)
  for (int c = tid; c < NH; c += blockDim.x) {
    float s = 0.f;
    for (int r = 0; r < TILE; ++r) s += __bfloat162float(D2[r * LDH + c]);
    atomicAdd(&A.grad[OFF_B2 + c], s);
  }
  // dH1 = dZ2 W2 (K = 128 outputs of layer 2), then dZ1
  const int m0 = warp * 16, g = lane >> 2, tq = lane & 3;
  float acc[16][4];
#pragma unroll
  for (int j = 0; j < 16; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
  for (int k0 = 0; k0 < NH; k0 += 16) {
    uint32_t a[4];
    load_a(a, D2, LDH, m0, k0, lane);
#pragma unroll
    for (int j = 0; j < 16; ++j) {
      uint32_t b[2];
      load_b(b, W2t, LDH, j * 8, k0, lane);
      mma16816(acc[j], a, b);
    }
  }
  __syncthreads();
  float *colsum = red;
  for (int c = tid; c < NH; c += blockDim.x) colsum[c] = 0.f;
  __syncthreads();
#pragma unroll
  for (int j = 0; j < 16; ++j) {
    const int col = j * 8 + 2 * tq;
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const int r = m0 + g + 8 * h;
      if (row0 + r < A.nb) {
        const long o = (long)(row0 + r) * NH + col;
        const bf16 d0 = __float2bfloat16(acc[j][2 * h] * gelu_grad_f(A.z1[o]));
        const bf16 d1 = __float2bfloat16(acc[j][2 * h + 1] * gelu_grad_f(A.z1[o + 1]));
        A.dz1[o] = d0;
        A.dz1[o + 1] = d1;
        atomicAdd(&colsum[col], __bfloat162float(d0));
        atomicAdd(&colsum[col + 1], __bfloat162float(d1));
      }
    }
  }
  __syncthreads();
  for (int c = tid; c < NH; c += blockDim.x) atomicAdd(&A.grad[OFF_B1 + c], colsum[c]);
}

size_t mlp_backward_smem() {
  return (size_t)(NH * LDH + TILE * LDH) * sizeof(bf16) + (size_t)(NOUT * NH + TILE * NOUT + NH) * sizeof(float);
}

// ---------------------------------------------------------------------------
// Weight gradient G[o][i] += sum_r D[r][o] * H[r][i] over a chunk of batch
// rows (tensor cores, K = batch): 8 warps, warp w owns outputs 16w..16w+15.
// ---------------------------------------------------------------------------
template <int NI>
__global__ void __launch_bounds__(256) k_mlp_wgrad(int nb, const bf16 *__restrict__ D, const bf16 *__restrict__ H,
                                                    float *__restrict__ G, int chunk) {
  constexpr int KT = 32;            // batch rows per shared-memory stage
  constexpr int LDK = KT + 8;
  __shared__ __align__(16) bf16 Ds[NH * LDK];   // Ds[o][r]
  __shared__ __align__(16) bf16 Hs[NI * LDK];   // Hs[i][r]
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int g = lane >> 2, tq = lane & 3;
  constexpr int NJ = NI / 8;
  float acc[NJ][4];
#pragma unroll
  for (int j = 0; j < NJ; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
  const int r0 = blockIdx.x * chunk, r1 = min(nb, r0 + chunk);
  for (int rb = r0; rb < r1; rb += KT) {
    __syncthreads();
    for (int t = tid; t < KT * NH; t += blockDim.x) {
      const int r = t / NH, o = t % NH;
      Ds[o * LDK + r] = (rb + r < r1) ? D[(long)(rb + r) * NH + o] : __float2bfloat16(0.f);
    }
    for (int t = tid; t < KT * NI; t += blockDim.x) {
      const int r = t / NI, i = t % NI;
      Hs[i * LDK + r] = (rb + r < r1) ? H[(long)(rb + r) * NI + i] : __float2bfloat16(0.f);
    }
    __syncthreads();
#pragma unroll
    for (int k0 = 0; k0 < KT; k0 += 16) {
      uint32_t a[4];
      load_a(a, Ds, LDK, warp * 16, k0, lane);
#pragma unroll
      for (int j = 0; j < NJ; ++j) {
        uint32_t b[2];
        load_b(b, Hs, LDK, j * 8, k0, lane);
        mma16816(acc[j], a, b);
      }
    }
  }
#pragma unroll
  for (int j = 0; j < NJ; ++j) {
    const int col = j * 8 + 2 * tq;
    const int o0 = warp * 16 + g;
    atomicAdd(&G[o0 * NI + col], acc[j][0]);
    atomicAdd(&G[o0 * NI + col + 1], acc[j][1]);
    atomicAdd(&G[(o0 + 8) * NI + col], acc[j][2]);
    atomicAdd(&G[(o0 + 8) * NI + col + 1], acc[j][3]);
  }
}

// Adam (FP32 masters) followed by the BF16 weight copies
__global__ void k_adam(float *__restrict__ p, const float *__restrict__ gr, float *__restrict__ m,
                       float *__restrict__ v, int n, float lr, float b1, float b2, float eps, float c1, float c2) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n; t += gridDim.x * blockDim.x) {
    const float g = gr[t];
    const float mm = b1 * m[t] + (1.f - b1) * g;
    const float vv = b2 * v[t] + (1.f - b2) * g * g;
    m[t] = mm;
    v[t] = vv;
    p[t] -= lr * (mm / c1) / (sqrtf(vv / c2) + eps);
  }
}
__global__ void k_refresh_bf16(const float *__restrict__ p, bf16 *__restrict__ w1b, bf16 *__restrict__ w2b,
                               bf16 *__restrict__ w2tb) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < NH * NIN + NH * NH; t += gridDim.x * blockDim.x) {
    if (t < NH * NIN) {
      w1b[t] = __float2bfloat16(p[t]);
    } else {
      const int q = t - NH * NIN, o = q / NH, i = q % NH;
      const bf16 v = __float2bfloat16(p[OFF_W2 + q]);
      w2b[q] = v;
      w2tb[i * NH + o] = v;
    }
  }
}

int mlp_nparam() { return NPARAM; }

void launch_mlp_refresh(cudaStream_t s, const float *params, bf16 *w1b, bf16 *w2b, bf16 *w2tb) {
  k_refresh_bf16<<<64, 256, 0, s>>>(params, w1b, w2b, w2tb);
}

// one optimisation step on a batch already staged in x (bf16) and t (fp32)
void launch_mlp_train_step(cudaStream_t s, const MlpTrainBuffers &B, int nb, int step, float lr) {
  cudaMemsetAsync(B.grad, 0, NPARAM * sizeof(float), s);
  cudaMemsetAsync(B.loss, 0, sizeof(float), s);
  launch_mlp_forward(s, B.x, nb, B.w1b, B.w2b, B.params, B.y, B.z1, B.z2, B.h1, B.h2, 1);
  MlpBwdArgs A{nb, B.y, B.t, B.z1, B.z2, B.h2, B.w2tb, B.params, B.dz1, B.dz2, B.grad, B.loss};
  k_mlp_backward<<<(nb + TILE - 1) / TILE, 128, mlp_backward_smem(), s>>>(A);
  const int chunk = 512;
  const int nchunk = (nb + chunk - 1) / chunk;
  k_mlp_wgrad<NH><<<nchunk, 256, 0, s>>>(nb, B.dz2, B.h1, B.grad + OFF_W2, chunk);
  k_mlp_wgrad<NIN><<<nchunk, 256, 0, s>>>(nb, B.dz1, B.x, B.grad, chunk);
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)step), c2 = 1.f - powf(b2, (float)step);
  k_adam<<<64, 256, 0, s>>>(B.params, B.grad, B.m, B.v, NPARAM, lr, b1, b2, 1e-8f, c1, c2);
  k_refresh_bf16<<<64, 256, 0, s>>>(B.params, B.w1b, B.w2b, B.w2tb);
}

// gradient only (for the check against the CPU reference)
void launch_mlp_grad(cudaStream_t s, const MlpTrainBuffers &B, int nb) {
  cudaMemsetAsync(B.grad, 0, NPARAM * sizeof(float), s);
  cudaMemsetAsync(B.loss, 0, sizeof(float), s);
  launch_mlp_forward(s, B.x, nb, B.w1b, B.w2b, B.params, B.y, B.z1, B.z2, B.h1, B.h2, 1);
  MlpBwdArgs A{nb, B.y, B.t, B.z1, B.z2, B.h2, B.w2tb, B.params, B.dz1, B.dz2, B.grad, B.loss};
  k_mlp_backward<<<(nb + TILE - 1) / TILE, 128, mlp_backward_smem(), s>>>(A);
  const int chunk = 512;
  const int nchunk = (nb + chunk - 1) / chunk;
  k_mlp_wgrad<NH><<<nchunk, 256, 0, s>>>(nb, B.dz2, B.h1, B.grad + OFF_W2, chunk);
  k_mlp_wgrad<NIN><<<nchunk, 256, 0, s>>>(nb, B.dz1, B.x, B.grad, chunk);
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

// batch of nb rows drawn with replacement by a counter-based hash of
// (seed, step, row) -- no host round trip between optimisation steps
__device__ __forceinline__ unsigned mix32(unsigned x) {
  x ^= x >> 16; x *= 0x7feb352dU; x ^= x >> 15; x *= 0x846ca68bU; x ^= x >> 16;
  return x;
}
__global__ void k_mlp_gather(int n, const bf16 *__restrict__ X, const float *__restrict__ T, int nb, unsigned seed,
                             int step, bf16 *__restrict__ bx, float *__restrict__ bt) {
  for (int r = blockIdx.x * (blockDim.x / 32) + (threadIdx.x >> 5); r < nb; r += gridDim.x * (blockDim.x / 32)) {
    const unsigned h = mix32(seed ^ mix32((unsigned)step * 0x9E3779B9U + (unsigned)r));
    const int src = (int)(h % (unsigned)n);
    const int lane = threadIdx.x & 31;
    // 96 bf16 = 48 words per row
    const uint32_t *xs = reinterpret_cast<const uint32_t *>(X + (long)src * NIN);
    uint32_t *xd = reinterpret_cast<uint32_t *>(bx + (long)r * NIN);
    for (int w = lane; w < NIN / 2; w += 32) xd[w] = xs[w];
    if (lane < NOUT) bt[(long)r * NOUT + lane] = T[(long)src * NOUT + lane];
  }
}
void launch_mlp_gather(cudaStream_t s, int n, const bf16 *X, const float *T, int nb, unsigned seed, int step, bf16 *bx,
                       float *bt) {
  k_mlp_gather<<<(nb + 7) / 8 < 1216 ? (nb + 7) / 8 : 1216, 256, 0, s>>>(n, X, T, nb, seed, step, bx, bt);
}

__global__ void k_f2bf(long n, const float *__restrict__ a, bf16 *__restrict__ b) {
  for (long q = blockIdx.x * (long)blockDim.x + threadIdx.x; q < n; q += (long)gridDim.x * blockDim.x)
    b[q] = __float2bfloat16(a[q]);
}
void launch_f2bf(cudaStream_t s, long n, const float *a, bf16 *b) { k_f2bf<<<608, 256, 0, s>>>(n, a, b); }

int mlp_set_smem_limits() {
  cudaError_t e1 = cudaFuncSetAttribute(k_mlp_forward<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)mlp_forward_smem());
  cudaError_t e2 = cudaFuncSetAttribute(k_mlp_forward<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)mlp_forward_smem());
  cudaError_t e3 = cudaFuncSetAttribute(k_mlp_backward, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)mlp_backward_smem());
  cudaError_t e4 = cudaFuncSetAttribute(k_mlp_infer, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)mlp_infer_smem());
  cudaError_t e5 = cudaFuncSetAttribute(k_mlp_infer_tc<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
  if (e5 == cudaSuccess)
    e5 = cudaFuncSetAttribute(k_mlp_infer_tc<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)TC_SMEM);
  return (e1 == cudaSuccess && e2 == cudaSuccess && e3 == cudaSuccess && e4 == cudaSuccess && e5 == cudaSuccess)
             ? 0
             : -1;
}

}  // namespace ibmk
