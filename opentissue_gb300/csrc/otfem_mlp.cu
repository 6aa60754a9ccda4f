// otfem_mlp.cu -- learned warm start for the matrix-free CG.
//
// No counterpart in the reference: fem_conjugate_gradients.h:44-46 starts CG
// from the previous velocity, which stays the fallback and the judge of the
// learned guess (CG always runs to the same relative residual from either).
//
// The network is node-wise: inputs per node are its velocity v, its velocity
// change of the previous step dv_prev, its external force, and the mean of
// the 9 entries of Re over the tets that contain it (18 inputs, normalised by
// per-input mean and standard deviation of the training set).  Three hidden
// layers of 64 with GELU (tanh form) and a linear output of 3 predict the
// change of dv from the previous step (normalised): the initial guess is
// v + dv_prev + prediction.
//
// All matrix products run on the tensor cores as BF16 mma.sync m16n8k16
// tiles with FP32 accumulation.  A warp owns 16 rows (nodes or samples);
// the FP32 accumulator tile of one layer, rounded to BF16, is exactly the A
// operand tile of the next, so activations stay in registers between layers.
// Training fuses forward, backward and the weight-gradient products for a
// chunk of 64 samples per CTA; Adam (Kingma & Ba, 2015) updates FP32 master
// weights and re-packs the BF16 operands.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

#include "otfem_internal.h"

// ---- layout ---------------------------------------------------------------
namespace otfem {
namespace {

constexpr int kIn = kFeatures;  // 18
constexpr int kInPad = 32;
constexpr int kHid = 64;
constexpr int kOut = 3;
// FP32 parameter vector, each layer as weight[out][in] then bias[out]
constexpr int kOffW1 = 0;
constexpr int kOffB1 = kOffW1 + kHid * kIn;
constexpr int kOffW2 = kOffB1 + kHid;
constexpr int kOffB2 = kOffW2 + kHid * kHid;
constexpr int kOffW3 = kOffB2 + kHid;
constexpr int kOffB3 = kOffW3 + kHid * kHid;
constexpr int kOffW4 = kOffB3 + kHid;
constexpr int kOffB4 = kOffW4 + kOut * kHid;
constexpr int kNumParams = kOffB4 + kOut;  // 9731
// normalisation: mean[18], std[18] of the inputs, mean[3], std[3] of the targets
constexpr int kNormMuX = 0, kNormSdX = kIn, kNormMuY = 2 * kIn, kNormSdY = 2 * kIn + kOut;
constexpr int kNumNorm = 2 * kIn + 2 * kOut;  // 42
static_assert(kNumParams + kNumNorm == OTFEM_MLP_STATE_SIZE, "state size");

// BF16 operand copies.  B operand of y = x W^T: element (k = in, n = out) at
// W[n][k], rows padded to K + 8 elements so the 8 row groups of a warp's
// fragment loads fall in different shared-memory banks.  The backward pass
// multiplies by W, whose B operand (k = out, n = in) is the transpose.
constexpr int kLd1 = kInPad + 8;  // W1 [64][40]
constexpr int kLdH = kHid + 8;    // W2, W3 [64][72], W4 [8][72], W2t, W3t [64][72]
constexpr int kLd4t = 16 + 8;     // W4t [64][24] (out padded to 16)
constexpr int kW1p = 0;
constexpr int kW2p = kW1p + kHid * kLd1;
constexpr int kW3p = kW2p + kHid * kLdH;
constexpr int kW4p = kW3p + kHid * kLdH;
constexpr int kFwdElems = kW4p + 8 * kLdH;
constexpr int kW2t = kFwdElems;
constexpr int kW3t = kW2t + kHid * kLdH;
constexpr int kW4t = kW3t + kHid * kLdH;
constexpr int kPackedElems = kW4t + kHid * kLd4t;
static_assert((kFwdElems * 2) % 16 == 0 && (kPackedElems * 2) % 16 == 0, "16-byte copies");

// training sample: inputs (kFeatureStride floats, 18 used), target (4 floats, 3 used)
constexpr int kTargetStride = 4;
constexpr int kTrainWarps = 4;
constexpr int kChunk = 16 * kTrainWarps;  // samples per CTA pass
constexpr int kLdR = kChunk + 8;          // row stride of the transposed chunk tiles
constexpr int kXs = kInPad + 4;           // row stride of the input staging
constexpr int kFeatWarps = 8;             // inference: 8 warps x 32 nodes per CTA

// ---- tensor-core building blocks ------------------------------------------
__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  __nv_bfloat162 h = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<uint32_t*>(&h);
}

__device__ __forceinline__ void mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// c[16 x 8NT] += a[16 x 16KT] * B, B element (k, n) at Bs[n * ld + k] (BF16,
// shared memory).  Fragment layouts (PTX ISA, mma.m16n8k16): lane = 4g + t;
// a[kt] = A(g, 16kt+2t..+1), A(g+8, ..), A(g, 16kt+8+2t..+1), A(g+8, ..);
// B pair (16kt+2t..+1, n = 8nt+g) and (16kt+8+2t..+1, n); c[nt] = C(g,
// 8nt+2t..+1), C(g+8, 8nt+2t..+1).
template <int KT, int NT>
__device__ __forceinline__ void warp_gemm(const uint32_t (&a)[KT][4], const __nv_bfloat16* Bs, int ld,
                                          float (&c)[NT][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const __nv_bfloat16* row = Bs + (8 * nt + g) * ld + 2 * t;
#pragma unroll
    for (int kt = 0; kt < KT; ++kt) {
      const uint32_t b0 = *reinterpret_cast<const uint32_t*>(row + 16 * kt);
      const uint32_t b1 = *reinterpret_cast<const uint32_t*>(row + 16 * kt + 8);
      mma_bf16(c[nt], a[kt], b0, b1);
    }
  }
}

// A fragments (16 x 8NT) of the BF16-rounded accumulator tile.
template <int NT>
__device__ __forceinline__ void c_to_a(const float (&c)[NT][4], uint32_t (&a)[NT / 2][4]) {
#pragma unroll
  for (int kt = 0; kt < NT / 2; ++kt) {
    a[kt][0] = pack_bf16(c[2 * kt][0], c[2 * kt][1]);
    a[kt][1] = pack_bf16(c[2 * kt][2], c[2 * kt][3]);
    a[kt][2] = pack_bf16(c[2 * kt + 1][0], c[2 * kt + 1][1]);
    a[kt][3] = pack_bf16(c[2 * kt + 1][2], c[2 * kt + 1][3]);
  }
}

// A fragments of rows 0..15 of a row-major FP32 tile (stride ld).
template <int KT>
__device__ __forceinline__ void load_a(const float* x, int ld, uint32_t (&a)[KT][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int kt = 0; kt < KT; ++kt) {
    const int c0 = 16 * kt + 2 * t;
    a[kt][0] = pack_bf16(x[g * ld + c0], x[g * ld + c0 + 1]);
    a[kt][1] = pack_bf16(x[(g + 8) * ld + c0], x[(g + 8) * ld + c0 + 1]);
    a[kt][2] = pack_bf16(x[g * ld + c0 + 8], x[g * ld + c0 + 9]);
    a[kt][3] = pack_bf16(x[(g + 8) * ld + c0 + 8], x[(g + 8) * ld + c0 + 9]);
  }
}

// A fragments (m-tile of rows m0..m0+15) of a row-major BF16 tile (stride ld).
template <int KT>
__device__ __forceinline__ void load_a_bf16(const __nv_bfloat16* x, int ld, int m0, uint32_t (&a)[KT][4]) {
  const int lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int kt = 0; kt < KT; ++kt) {
    const int c0 = 16 * kt + 2 * t;
    a[kt][0] = *reinterpret_cast<const uint32_t*>(x + (m0 + g) * ld + c0);
    a[kt][1] = *reinterpret_cast<const uint32_t*>(x + (m0 + g + 8) * ld + c0);
    a[kt][2] = *reinterpret_cast<const uint32_t*>(x + (m0 + g) * ld + c0 + 8);
    a[kt][3] = *reinterpret_cast<const uint32_t*>(x + (m0 + g + 8) * ld + c0 + 8);
  }
}

// GELU, tanh form: 0.5 z (1 + tanh(u)), u = sqrt(2/pi) (z + 0.044715 z^3).
// With 0.5 (1 + tanh(u)) = 1 / (1 + exp(-2u)) (the logistic function of 2u)
// it is z s with s = 1 / (1 + exp(-2u)), one exponential and one division;
// the derivative is s + z s (1 - s) 2 u'.  Large |u| saturate cleanly
// (exp -> inf gives s = 0, exp -> 0 gives s = 1).
constexpr float kGeluC = 0.7978845608028654f, kGeluA = 0.044715f;
__device__ __forceinline__ float gelu_logistic(float z) {
  const float u = kGeluC * (z + kGeluA * z * z * z);
  return __fdividef(1.f, 1.f + __expf(-2.f * u));
}
__device__ __forceinline__ float gelu(float z) { return z * gelu_logistic(z); }
__device__ __forceinline__ float gelu_grad(float z) {
  const float s = gelu_logistic(z);
  return s + z * s * (1.f - s) * (2.f * kGeluC) * (1.f + 3.f * kGeluA * z * z);
}

// Bias of columns 8nt+2t..+1 into both rows of the accumulator tile.
template <int NT>
__device__ __forceinline__ void init_bias(const float* b, int n_valid, float (&c)[NT][4]) {
  const int t = threadIdx.x & 3;
#pragma unroll
  for (int nt = 0; nt < NT; ++nt) {
    const int n = 8 * nt + 2 * t;
    const float b0 = n < n_valid ? b[n] : 0.f, b1 = n + 1 < n_valid ? b[n + 1] : 0.f;
    c[nt][0] = c[nt][2] = b0;
    c[nt][1] = c[nt][3] = b1;
  }
}

// Forward pass of one warp's 16 rows (normalised inputs in x, stride kXs) to
// the 3 outputs (accumulator tile columns 0..2).
__device__ __forceinline__ void mlp_forward16(const float* x, const __nv_bfloat16* Wf, const float* params,
                                              float (&out)[1][4]) {
  uint32_t a0[2][4];
  load_a<2>(x, kXs, a0);
  float z[8][4];
  uint32_t a[4][4];
  init_bias<8>(params + kOffB1, kHid, z);
  warp_gemm<2, 8>(a0, Wf + kW1p, kLd1, z);
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int j = 0; j < 4; ++j) z[nt][j] = gelu(z[nt][j]);
  c_to_a<8>(z, a);
  init_bias<8>(params + kOffB2, kHid, z);
  warp_gemm<4, 8>(a, Wf + kW2p, kLdH, z);
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int j = 0; j < 4; ++j) z[nt][j] = gelu(z[nt][j]);
  c_to_a<8>(z, a);
  init_bias<8>(params + kOffB3, kHid, z);
  warp_gemm<4, 8>(a, Wf + kW3p, kLdH, z);
#pragma unroll
  for (int nt = 0; nt < 8; ++nt)
#pragma unroll
    for (int j = 0; j < 4; ++j) z[nt][j] = gelu(z[nt][j]);
  c_to_a<8>(z, a);
  init_bias<1>(params + kOffB4, kOut, out);
  warp_gemm<4, 1>(a, Wf + kW4p, kLdH, out);
}

// Copies `bytes` (a multiple of 16) from global to shared memory.
__device__ __forceinline__ void copy16(void* dst, const void* src, int bytes) {
  uint4* d = reinterpret_cast<uint4*>(dst);
  const uint4* s = reinterpret_cast<const uint4*>(src);
  for (int k = threadIdx.x; k < bytes / 16; k += blockDim.x) d[k] = s[k];
}

// ---- kernels ---------------------------------------------------------------
struct FeatureArgs {
  int N, T;
  const unsigned char* fixed;
  const double* v;
  const float4* dv_last;
  const double* fext;
  const int* inc_ptr;
  const int* inc_ent;
  const float* re_f;       // 9 x T (SoA); used when tile_f is null
  const float* tile_f;     // the tets' rotations as quaternions (tile words 4..7), or null
  int tile_tets;
  unsigned long long tile_magic;
  const float4* quat_g;    // or the quaternions in the w of the mixed force entries (g_f), or null
  float* features;         // N x kFeatureStride or null
  float4* warm_dv;         // null: features only
  const __nv_bfloat16* packed;
  const float* params;
  const float* norm;
};

// Network inputs of every node and, with a.warm_dv, the learned initial
// guess.  8 warps per CTA, 32 nodes per warp (one per lane for the inputs,
// two 16-row tiles for the network).
__global__ void __launch_bounds__(32 * kFeatWarps, 3) k_node_features(FeatureArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16* Wf = reinterpret_cast<__nv_bfloat16*>(smem);
  float* xs_all = reinterpret_cast<float*>(smem + kFwdElems * sizeof(__nv_bfloat16));
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  float* xs = xs_all + warp * 32 * kXs;
  float* os = xs_all + kFeatWarps * 32 * kXs + warp * 32 * 4;
  const bool predict = a.warm_dv != nullptr;
  if (predict) copy16(Wf, a.packed, kFwdElems * sizeof(__nv_bfloat16));
  const int i = (blockIdx.x * kFeatWarps + warp) * 32 + lane;
  float f[kIn];
#pragma unroll
  for (int k = 0; k < kIn; ++k) f[k] = 0.f;
  if (i < a.N) {
    const float4 d = a.dv_last[i];
    for (int c = 0; c < 3; ++c) {
      f[c] = float(a.v[3L * i + c]);
      f[6 + c] = float(a.fext[3L * i + c]);
    }
    f[3] = d.x, f[4] = d.y, f[5] = d.z;
    const int q0 = a.inc_ptr[i], q1 = a.inc_ptr[i + 1];
    if (a.quat_g || a.tile_f) {
      // the tets' rotations from their quaternions (the FP32 rotation of the
      // matrix-free solvers is rebuilt the same way), four tets at a time:
      // their incidence entries, then their quaternions, are loaded ahead of
      // the sums so that the dependent gathers overlap
      for (int q = q0; q < q1; q += 4) {
        int tq[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) tq[k] = q + k < q1 ? a.inc_ent[q + k] >> 2 : -1;
        float4 qt[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          const int t = tq[k];
          qt[k] = t < 0 ? make_float4(0.f, 0.f, 0.f, 1.f)
                  : a.quat_g ? make_float4(a.quat_g[4L * t].w, a.quat_g[4L * t + 1].w, a.quat_g[4L * t + 2].w,
                                           a.quat_g[4L * t + 3].w)
                             : tile_quaternion(a.tile_f, a.tile_tets, tile_of(t, a.tile_magic), t);
        }
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (tq[k] < 0) break;
          float R[9];
          quaternion_to_rotation(qt[k], R);
#pragma unroll
          for (int c = 0; c < 9; ++c) f[9 + c] += R[c];
        }
      }
    } else {
      for (int q = q0; q < q1; ++q) {
        const int t = a.inc_ent[q] >> 2;
#pragma unroll
        for (int k = 0; k < 9; ++k) f[9 + k] += a.re_f[long(k) * a.T + t];
      }
    }
    if (q1 > q0) {
      const float inv = 1.f / float(q1 - q0);
#pragma unroll
      for (int k = 0; k < 9; ++k) f[9 + k] *= inv;
    }
    if (a.features) {
      float* o = a.features + long(i) * kFeatureStride;
#pragma unroll
      for (int k = 0; k < kIn; ++k) o[k] = f[k];
      o[kIn] = 0.f;
      o[kIn + 1] = 0.f;
    }
  }
  if (!predict) return;
  // normalised inputs of this lane's node as row `lane` of the staging tile
#pragma unroll
  for (int k = 0; k < kInPad; ++k)
    xs[lane * kXs + k] = (k < kIn && i < a.N) ? (f[k] - a.norm[kNormMuX + k]) / a.norm[kNormSdX + k] : 0.f;
  __syncthreads();  // weights staged, inputs visible to the warp
  const int g = lane >> 2, t = lane & 3;
#pragma unroll
  for (int mt = 0; mt < 2; ++mt) {
    float out[1][4];
    mlp_forward16(xs + 16 * mt * kXs, Wf, a.params, out);
    if (2 * t < kOut) {
      os[(16 * mt + g) * 4 + 2 * t] = out[0][0];
      os[(16 * mt + g + 8) * 4 + 2 * t] = out[0][2];
    }
    if (2 * t + 1 < kOut) {
      os[(16 * mt + g) * 4 + 2 * t + 1] = out[0][1];
      os[(16 * mt + g + 8) * 4 + 2 * t + 1] = out[0][3];
    }
  }
  __syncwarp();
  if (i < a.N) {
    float4 w = make_float4(0.f, 0.f, 0.f, 0.f);
    if (!a.fixed[i]) {
      w.x = f[3] + os[lane * 4 + 0] * a.norm[kNormSdY + 0] + a.norm[kNormMuY + 0];
      w.y = f[4] + os[lane * 4 + 1] * a.norm[kNormSdY + 1] + a.norm[kNormMuY + 1];
      w.z = f[5] + os[lane * 4 + 2] * a.norm[kNormSdY + 2] + a.norm[kNormMuY + 2];
    }
    a.warm_dv[i] = w;
  }
}

// One 1-ring mean pass over the network's correction c = warm - dv_prev:
// c_i <- mean over the tets t containing i of the mean of c over t's nodes
// (fixed nodes contribute 0); out = dv_prev + c for free nodes, 0 for fixed.
__global__ void k_smooth_correction(int N, const unsigned char* __restrict__ fixed, const int* __restrict__ inc_ptr,
                                    const int* __restrict__ inc_ent, const int4* __restrict__ tets,
                                    const float4* __restrict__ dv_prev, const float4* in, float4* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N) return;
  if (fixed[i]) {
    out[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    return;
  }
  float sx = 0.f, sy = 0.f, sz = 0.f;
  const int q0 = inc_ptr[i], q1 = inc_ptr[i + 1];
  for (int q = q0; q < q1; ++q) {
    const int4 n = tets[inc_ent[q] >> 2];
    const int nn[4] = {n.x, n.y, n.z, n.w};
#pragma unroll
    for (int k = 0; k < 4; ++k) {
      if (fixed[nn[k]]) continue;
      const float4 w = in[nn[k]], d = dv_prev[nn[k]];
      sx += w.x - d.x, sy += w.y - d.y, sz += w.z - d.z;
    }
  }
  const float inv = q1 > q0 ? 1.f / float(4 * (q1 - q0)) : 0.f;
  const float4 d = dv_prev[i];
  out[i] = make_float4(d.x + sx * inv, d.y + sy * inv, d.z + sz * inv, 0.f);
}

struct TrainArgs {
  const float* X;      // samples x kFeatureStride (raw inputs)
  const float* Y;      // samples x kTargetStride (raw targets)
  const int* perm;     // sample order
  long long off;       // first position in perm of this batch
  int batch;           // samples in this batch
  float scale;         // 2 / (3 * batch): d loss / d output = scale * (output - target)
  int grad;            // 0: loss only
  const float* norm;
  const float* params;
  const __nv_bfloat16* packed;
  float* gradient;     // kNumParams (accumulated)
  double* loss;        // sum of squared normalised errors (accumulated)
};

// Shared-memory layout of the training kernel.
struct TrainSmem {
  static constexpr size_t wf = 0;
  static constexpr size_t wb = wf + kFwdElems * 2;
  static constexpr size_t xs = wb + (kPackedElems - kFwdElems) * 2;
  static constexpr size_t gd = xs + kTrainWarps * 16 * kXs * 4;      // GELU derivatives [3][64][64] FP32
  static constexpr size_t ht0 = gd + 3 * kChunk * kHid * 4;          // inputs^T [32][kLdR] BF16
  static constexpr size_t ht = ht0 + kInPad * kLdR * 2;              // activations^T [3][64][kLdR]
  static constexpr size_t dz = ht + 3 * kHid * kLdR * 2;             // pre-activation grads^T [3][64][kLdR]
  static constexpr size_t dz4 = dz + 3 * kHid * kLdR * 2;            // output grads^T [16][kLdR]
  static constexpr size_t db = dz4 + 16 * kLdR * 2;                  // bias grads [3*64 + 3]
  static constexpr size_t lossp = db + (3 * kHid + 4) * 4;           // loss partial (double)
  static constexpr size_t bytes = lossp + 16;
};

// Forward, backward and weight gradients of `batch` samples.  Each CTA takes
// chunks of 64 samples (16 per warp), accumulates its weight gradients in
// registers and adds them to a.gradient once at the end.
__global__ void __launch_bounds__(32 * kTrainWarps, 1) k_mlp_train(TrainArgs a) {
  extern __shared__ __align__(16) unsigned char smem[];
  __nv_bfloat16* Wf = reinterpret_cast<__nv_bfloat16*>(smem + TrainSmem::wf);
  __nv_bfloat16* Wb = reinterpret_cast<__nv_bfloat16*>(smem + TrainSmem::wb);
  float* gd = reinterpret_cast<float*>(smem + TrainSmem::gd);
  __nv_bfloat16* ht0 = reinterpret_cast<__nv_bfloat16*>(smem + TrainSmem::ht0);
  __nv_bfloat16* ht = reinterpret_cast<__nv_bfloat16*>(smem + TrainSmem::ht);
  __nv_bfloat16* dz = reinterpret_cast<__nv_bfloat16*>(smem + TrainSmem::dz);
  __nv_bfloat16* dz4 = reinterpret_cast<__nv_bfloat16*>(smem + TrainSmem::dz4);
  float* db = reinterpret_cast<float*>(smem + TrainSmem::db);
  double* lossp = reinterpret_cast<double*>(smem + TrainSmem::lossp);
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31, g = lane >> 2, t = lane & 3;
  float* xs = reinterpret_cast<float*>(smem + TrainSmem::xs) + warp * 16 * kXs;
  copy16(Wf, a.packed, kPackedElems * 2);  // forward and backward operands are contiguous
  for (int k = threadIdx.x; k < 16 * kLdR; k += blockDim.x) dz4[k] = __float2bfloat16(0.f);
  for (int k = threadIdx.x; k < 3 * kHid + 4; k += blockDim.x) db[k] = 0.f;
  if (threadIdx.x == 0) *lossp = 0.0;
  float acc1[4][4], acc2[8][4], acc3[8][4], acc4[2][4];
#pragma unroll
  for (int n = 0; n < 8; ++n)
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      acc2[n][j] = acc3[n][j] = 0.f;
      if (n < 4) acc1[n][j] = 0.f;
      if (n < 2) acc4[n][j] = 0.f;
    }
  float my_loss = 0.f;
  __syncthreads();
  const int chunks = (a.batch + kChunk - 1) / kChunk;
  for (int ch = blockIdx.x; ch < chunks; ch += gridDim.x) {
    const int r0 = 16 * warp;  // this warp's rows within the chunk
    // inputs: lanes 0..15 load one sample each
    if (lane < 16) {
      const int pos = ch * kChunk + r0 + lane;
      const bool valid = pos < a.batch;
      const float* x = valid ? a.X + long(a.perm[a.off + pos]) * kFeatureStride : nullptr;
#pragma unroll
      for (int k = 0; k < kInPad; ++k) {
        const float xn = (valid && k < kIn) ? (x[k] - a.norm[kNormMuX + k]) / a.norm[kNormSdX + k] : 0.f;
        xs[lane * kXs + k] = xn;
        ht0[k * kLdR + r0 + lane] = __float2bfloat16(xn);
      }
    }
    __syncwarp();
    // forward, keeping GELU'(z) and the activations (transposed) for backward
    uint32_t a0[2][4];
    load_a<2>(xs, kXs, a0);
    float z[8][4];
    uint32_t ah[4][4];
    const float* bias[3] = {a.params + kOffB1, a.params + kOffB2, a.params + kOffB3};
#pragma unroll
    for (int l = 0; l < 3; ++l) {
      init_bias<8>(bias[l], kHid, z);
      if (l == 0) warp_gemm<2, 8>(a0, Wf + kW1p, kLd1, z);
      else warp_gemm<4, 8>(ah, Wf + (l == 1 ? kW2p : kW3p), kLdH, z);
      float* G = gd + l * kChunk * kHid;
      __nv_bfloat16* H = ht + l * kHid * kLdR;
#pragma unroll
      for (int nt = 0; nt < 8; ++nt)
#pragma unroll
        for (int j = 0; j < 4; ++j) {
          const int r = r0 + g + (j >= 2 ? 8 : 0), c = 8 * nt + 2 * t + (j & 1);
          G[r * kHid + c] = gelu_grad(z[nt][j]);
          z[nt][j] = gelu(z[nt][j]);
          H[c * kLdR + r] = __float2bfloat16(z[nt][j]);
        }
      c_to_a<8>(z, ah);
    }
    float y4[1][4];
    init_bias<1>(a.params + kOffB4, kOut, y4);
    warp_gemm<4, 1>(ah, Wf + kW4p, kLdH, y4);
    // output error: rows g, g+8; columns 2t, 2t+1
    float d4[4];
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const int r = r0 + g + (j >= 2 ? 8 : 0), c = 2 * t + (j & 1);
      const int pos = ch * kChunk + r;
      float dj = 0.f;
      if (c < kOut && pos < a.batch) {
        const float y = (a.Y[long(a.perm[a.off + pos]) * kTargetStride + c] - a.norm[kNormMuY + c]) /
                        a.norm[kNormSdY + c];
        const float e = y4[0][j] - y;
        my_loss += e * e;
        dj = a.scale * e;
      }
      d4[j] = dj;
      if (c < 8) dz4[c * kLdR + r] = __float2bfloat16(dj);
    }
    if (a.grad) {
      {
        // output bias gradient: columns 2t, 2t+1 summed over the 16 rows
        float s0 = d4[0] + d4[2], s1 = d4[1] + d4[3];
#pragma unroll
        for (int o = 4; o < 32; o <<= 1) {
          s0 += __shfl_xor_sync(0xffffffffu, s0, o);
          s1 += __shfl_xor_sync(0xffffffffu, s1, o);
        }
        if (g == 0) {
          if (2 * t < kOut) atomicAdd(&db[3 * kHid + 2 * t], s0);
          if (2 * t + 1 < kOut) atomicAdd(&db[3 * kHid + 2 * t + 1], s1);
        }
      }
      // backward through the hidden layers: dz_l = (dz_{l+1} W_{l+1}) * GELU'(z_l)
      uint32_t ad[4][4];
      {
        uint32_t a4[1][4];
        a4[0][0] = pack_bf16(d4[0], d4[1]);
        a4[0][1] = pack_bf16(d4[2], d4[3]);
        a4[0][2] = 0u;
        a4[0][3] = 0u;
        float dh[8][4];
#pragma unroll
        for (int nt = 0; nt < 8; ++nt)
#pragma unroll
          for (int j = 0; j < 4; ++j) dh[nt][j] = 0.f;
        warp_gemm<1, 8>(a4, Wb + (kW4t - kFwdElems), kLd4t, dh);
#pragma unroll
        for (int l = 2; l >= 0; --l) {
          const float* G = gd + l * kChunk * kHid;
          __nv_bfloat16* D = dz + l * kHid * kLdR;
#pragma unroll
          for (int nt = 0; nt < 8; ++nt) {
            float s0 = 0.f, s1 = 0.f;
#pragma unroll
            for (int j = 0; j < 4; ++j) {
              const int r = r0 + g + (j >= 2 ? 8 : 0), c = 8 * nt + 2 * t + (j & 1);
              dh[nt][j] *= G[r * kHid + c];
              D[c * kLdR + r] = __float2bfloat16(dh[nt][j]);
            }
            s0 = dh[nt][0] + dh[nt][2];
            s1 = dh[nt][1] + dh[nt][3];
#pragma unroll
            for (int o = 4; o < 32; o <<= 1) {
              s0 += __shfl_xor_sync(0xffffffffu, s0, o);
              s1 += __shfl_xor_sync(0xffffffffu, s1, o);
            }
            if (g == 0) {
              atomicAdd(&db[l * kHid + 8 * nt + 2 * t], s0);
              atomicAdd(&db[l * kHid + 8 * nt + 2 * t + 1], s1);
            }
          }
          if (l > 0) {
            c_to_a<8>(dh, ad);
#pragma unroll
            for (int nt = 0; nt < 8; ++nt)
#pragma unroll
              for (int j = 0; j < 4; ++j) dh[nt][j] = 0.f;
            warp_gemm<4, 8>(ad, Wb + (l == 2 ? kW3t : kW2t) - kFwdElems, kLdH, dh);
          }
        }
      }
    }
    __syncthreads();  // the chunk's transposed tiles are complete
    if (a.grad) {
      // dW_l[o][i] = sum_r dz_l[r][o] h_{l-1}[r][i]: A = dz^T (o x r), B = (r, i) at h^T[i][r]
      uint32_t am[4][4];
      load_a_bf16<4>(dz + 0 * kHid * kLdR, kLdR, 16 * warp, am);
      warp_gemm<4, 4>(am, ht0, kLdR, acc1);
      load_a_bf16<4>(dz + 1 * kHid * kLdR, kLdR, 16 * warp, am);
      warp_gemm<4, 8>(am, ht + 0 * kHid * kLdR, kLdR, acc2);
      load_a_bf16<4>(dz + 2 * kHid * kLdR, kLdR, 16 * warp, am);
      warp_gemm<4, 8>(am, ht + 1 * kHid * kLdR, kLdR, acc3);
      load_a_bf16<4>(dz4, kLdR, 0, am);
      warp_gemm<4, 2>(am, ht + 2 * kHid * kLdR + 16 * warp * kLdR, kLdR, acc4);
    }
    __syncthreads();  // before the next chunk overwrites the tiles
  }
  // loss and gradients of this CTA
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) my_loss += __shfl_xor_sync(0xffffffffu, my_loss, o);
  if (lane == 0) atomicAdd(lossp, double(my_loss));
  __syncthreads();
  if (threadIdx.x == 0) atomicAdd(a.loss, *lossp);
  if (!a.grad) return;
#pragma unroll
  for (int j = 0; j < 4; ++j) {
    const int o = 16 * warp + g + (j >= 2 ? 8 : 0);
#pragma unroll
    for (int nt = 0; nt < 8; ++nt) {
      const int i = 8 * nt + 2 * t + (j & 1);
      if (nt < 4 && i < kIn) atomicAdd(&a.gradient[kOffW1 + o * kIn + i], acc1[nt][j]);
      atomicAdd(&a.gradient[kOffW2 + o * kHid + i], acc2[nt][j]);
      atomicAdd(&a.gradient[kOffW3 + o * kHid + i], acc3[nt][j]);
    }
    const int o4 = g + (j >= 2 ? 8 : 0);
#pragma unroll
    for (int n2 = 0; n2 < 2; ++n2) {
      const int i = 8 * (2 * warp + n2) + 2 * t + (j & 1);
      if (o4 < kOut) atomicAdd(&a.gradient[kOffW4 + o4 * kHid + i], acc4[n2][j]);
    }
  }
  for (int k = threadIdx.x; k < 3 * kHid + kOut; k += blockDim.x) {
    const int off = k < kHid ? kOffB1 + k : k < 2 * kHid ? kOffB2 + k - kHid : k < 3 * kHid ? kOffB3 + k - 2 * kHid
                                                                                           : kOffB4 + k - 3 * kHid;
    atomicAdd(&a.gradient[off], db[k]);
  }
}

// BF16 operand copies of the FP32 parameters (padding stays zero).
__global__ void k_pack_params(const float* __restrict__ p, __nv_bfloat16* packed) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kNumParams) return;
  const __nv_bfloat16 w = __float2bfloat16(p[k]);
  if (k < kOffB1) {
    const int o = (k - kOffW1) / kIn, i = (k - kOffW1) % kIn;
    packed[kW1p + o * kLd1 + i] = w;
  } else if (k >= kOffW2 && k < kOffB2) {
    const int o = (k - kOffW2) / kHid, i = (k - kOffW2) % kHid;
    packed[kW2p + o * kLdH + i] = w;
    packed[kW2t + i * kLdH + o] = w;
  } else if (k >= kOffW3 && k < kOffB3) {
    const int o = (k - kOffW3) / kHid, i = (k - kOffW3) % kHid;
    packed[kW3p + o * kLdH + i] = w;
    packed[kW3t + i * kLdH + o] = w;
  } else if (k >= kOffW4 && k < kOffB4) {
    const int o = (k - kOffW4) / kHid, i = (k - kOffW4) % kHid;
    packed[kW4p + o * kLdH + i] = w;
    packed[kW4t + i * kLd4t + o] = w;
  }
}

// Adam (Kingma & Ba 2015): m = b1 m + (1-b1) g, v = b2 v + (1-b2) g^2,
// p -= lr (m / c1) / (sqrt(v / c2) + eps) with c1 = 1 - b1^t, c2 = 1 - b2^t.
// Clears the gradient.
__global__ void k_adam(float* p, float* grad, float* m, float* v, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= kNumParams) return;
  const float gk = grad[k];
  const float mk = b1 * m[k] + (1.f - b1) * gk;
  const float vk = b2 * v[k] + (1.f - b2) * gk * gk;
  m[k] = mk;
  v[k] = vk;
  p[k] -= lr * (mk / c1) / (sqrtf(vk / c2) + eps);
  grad[k] = 0.f;
}

// Appends the free nodes of a step (features and target dv - dv_prev) to the
// training set; each node is kept when its hash is below `keep`.
__global__ void k_append_samples(int N, const unsigned char* fixed, const float* features, const float4* dv_last,
                                 float* X, float* Y, unsigned long long* count, long long cap, unsigned keep,
                                 unsigned long long seed) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= N || fixed[i]) return;
  unsigned long long h = seed + 0x9e3779b97f4a7c15ull * (unsigned long long)(i + 1);
  h = (h ^ (h >> 30)) * 0xbf58476d1ce4e5b9ull;
  h = (h ^ (h >> 27)) * 0x94d049bb133111ebull;
  h ^= h >> 31;
  if (unsigned(h >> 32) > keep) return;
  const unsigned long long slot = atomicAdd(count, 1ull);
  if ((long long)slot >= cap) return;
  const float* f = features + long(i) * kFeatureStride;
  float* x = X + (long long)slot * kFeatureStride;
  for (int k = 0; k < kFeatureStride; ++k) x[k] = f[k];
  const float4 d = dv_last[i];
  float* y = Y + (long long)slot * kTargetStride;
  y[0] = d.x - f[3];
  y[1] = d.y - f[4];
  y[2] = d.z - f[5];
  y[3] = 0.f;
}

// Column sums and sums of squares (FP64) of the first `rows` samples: 18
// inputs then 3 targets.
__global__ void k_column_moments(const float* X, const float* Y, long long rows, double* out) {
  __shared__ double s[2 * (kIn + kOut)];
  for (int k = threadIdx.x; k < 2 * (kIn + kOut); k += blockDim.x) s[k] = 0.0;
  __syncthreads();
  double loc[2 * (kIn + kOut)];
  for (int k = 0; k < 2 * (kIn + kOut); ++k) loc[k] = 0.0;
  for (long long r = blockIdx.x * (long long)blockDim.x + threadIdx.x; r < rows; r += (long long)gridDim.x * blockDim.x) {
    for (int k = 0; k < kIn; ++k) {
      const double x = X[r * kFeatureStride + k];
      loc[k] += x;
      loc[kIn + kOut + k] += x * x;
    }
    for (int k = 0; k < kOut; ++k) {
      const double y = Y[r * kTargetStride + k];
      loc[kIn + k] += y;
      loc[2 * kIn + kOut + k] += y * y;
    }
  }
  for (int k = 0; k < 2 * (kIn + kOut); ++k) atomicAdd(&s[k], loc[k]);
  __syncthreads();
  for (int k = threadIdx.x; k < 2 * (kIn + kOut); k += blockDim.x) atomicAdd(&out[k], s[k]);
}

// splitmix64 (Steele, Lea & Flood 2014)
uint64_t splitmix64(uint64_t& s) {
  uint64_t z = (s += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
double uniform01(uint64_t& s) { return double(splitmix64(s) >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace
}  // namespace otfem

using namespace otfem;

struct otfem_mlp_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  float* params = nullptr;
  float* grad = nullptr;
  float* adam_m = nullptr;
  float* adam_v = nullptr;
  float* norm = nullptr;
  __nv_bfloat16* packed = nullptr;
  float* X = nullptr;
  float* Y = nullptr;
  int* perm = nullptr;
  unsigned long long* count = nullptr;  // device sample counter
  double* scratch = nullptr;            // moments / loss
  long long cap = 0;
  long long adam_t = 0;
  int num_sms = 0;
};

namespace otfem {
namespace {

int mlp_fail(int code, const std::string& msg) { return record_error(code, msg); }
int mlp_cuda(cudaError_t e, const char* what) {
  return record_error(OTFEM_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}
#define MLP_CUDA(call)                                  \
  do {                                                  \
    cudaError_t e_ = (call);                            \
    if (e_ != cudaSuccess) return mlp_cuda(e_, #call);  \
  } while (0)

bool attributes_set = false;
cudaError_t set_attributes() {
  if (attributes_set) return cudaSuccess;
  cudaError_t e = cudaFuncSetAttribute(k_mlp_train, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                       int(TrainSmem::bytes));
  if (e != cudaSuccess) return e;
  const int feat_smem = kFwdElems * 2 + kFeatWarps * 32 * (kXs + 4) * 4;
  e = cudaFuncSetAttribute(k_node_features, cudaFuncAttributeMaxDynamicSharedMemorySize, feat_smem);
  if (e == cudaSuccess) attributes_set = true;
  return e;
}

cudaError_t pack(otfem_mlp_s* m) {
  k_pack_params<<<(kNumParams + 255) / 256, 256, 0, m->stream>>>(m->params, m->packed);
  return cudaGetLastError();
}

// Runs the training kernel over `batch` samples of perm from `off`.
cudaError_t run_train_kernel(otfem_mlp_s* m, const float* X, const float* Y, const int* perm, long long off,
                             int batch, bool grad) {
  TrainArgs a;
  a.X = X;
  a.Y = Y;
  a.perm = perm;
  a.off = off;
  a.batch = batch;
  a.scale = 2.f / (3.f * float(batch));
  a.grad = grad ? 1 : 0;
  a.norm = m->norm;
  a.params = m->params;
  a.packed = m->packed;
  a.gradient = m->grad;
  a.loss = m->scratch;
  int chunks = (batch + kChunk - 1) / kChunk;
  int grid = std::max(1, std::min(chunks, m->num_sms));
  k_mlp_train<<<grid, 32 * kTrainWarps, TrainSmem::bytes, m->stream>>>(a);
  return cudaGetLastError();
}

}  // namespace

cudaError_t launch_node_features(Context& c, bool predict) {
  if (predict && !c.mlp) return cudaErrorInvalidValue;
  if (!c.features && !predict) return cudaSuccess;
  cudaError_t e = set_attributes();
  if (e != cudaSuccess) return e;
  FeatureArgs a;
  a.N = c.N;
  a.T = c.T;
  a.fixed = c.fixed;
  a.v = c.v;
  a.dv_last = c.dv_last;
  a.fext = c.fext;
  a.inc_ptr = c.inc_ptr;
  a.inc_ent = c.inc_ent;
  a.re_f = c.re_f;
  a.tile_f = c.tile_f;
  a.tile_tets = c.tile_tets;
  a.tile_magic = c.tile_magic;
  a.quat_g = nullptr;  // the tile words: measured faster than the force entries' w lanes
  a.features = c.collect ? c.features : nullptr;
  a.warm_dv = predict ? c.warm_dv : nullptr;
  a.packed = predict ? c.mlp->packed : nullptr;
  a.params = predict ? c.mlp->params : nullptr;
  a.norm = predict ? c.mlp->norm : nullptr;
  const int per_cta = 32 * kFeatWarps;
  const int grid = std::max(1, (c.N + per_cta - 1) / per_cta);
  const int smem = predict ? kFwdElems * 2 + kFeatWarps * 32 * (kXs + 4) * 4 : 0;
  k_node_features<<<grid, per_cta, smem, c.stream>>>(a);
  if (!predict || c.warm_smoothing <= 0 || !c.warm_tmp) return cudaGetLastError();
  const int nb = std::max(1, (c.N + 255) / 256);
  float4* src = c.warm_dv;
  float4* dst = c.warm_tmp;
  for (int k = 0; k < c.warm_smoothing; ++k) {
    k_smooth_correction<<<nb, 256, 0, c.stream>>>(c.N, c.fixed, c.inc_ptr, c.inc_ent, c.tets, c.dv_last, src, dst);
    std::swap(src, dst);
  }
  if (src != c.warm_dv) {
    e = cudaMemcpyAsync(c.warm_dv, src, sizeof(float4) * size_t(c.N), cudaMemcpyDeviceToDevice, c.stream);
    if (e != cudaSuccess) return e;
  }
  return cudaGetLastError();
}

}  // namespace otfem

extern "C" {

int otfem_mlp_create(int64_t capacity, uint64_t seed, otfem_mlp* out) {
  if (!out || capacity < 0) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  *out = nullptr;
  otfem_mlp_s* m = new otfem_mlp_s();
  auto bail = [&](cudaError_t e, const char* what) {
    otfem_mlp_destroy(m);
    return mlp_cuda(e, what);
  };
  cudaError_t e;
  if ((e = cudaGetDevice(&m->device)) != cudaSuccess) return bail(e, "cudaGetDevice");
  if ((e = cudaDeviceGetAttribute(&m->num_sms, cudaDevAttrMultiProcessorCount, m->device)) != cudaSuccess)
    return bail(e, "cudaDeviceGetAttribute");
  if ((e = cudaStreamCreateWithFlags(&m->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return bail(e, "cudaStreamCreate");
  if ((e = set_attributes()) != cudaSuccess) return bail(e, "cudaFuncSetAttribute");
  m->cap = capacity;
  const size_t nc = size_t(std::max<int64_t>(capacity, 1));
  if ((e = cudaMalloc(&m->params, sizeof(float) * kNumParams)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->grad, sizeof(float) * kNumParams)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->adam_m, sizeof(float) * kNumParams)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->adam_v, sizeof(float) * kNumParams)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->norm, sizeof(float) * kNumNorm)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->packed, sizeof(__nv_bfloat16) * kPackedElems)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->X, sizeof(float) * kFeatureStride * nc)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->Y, sizeof(float) * kTargetStride * nc)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->perm, sizeof(int) * nc)) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->count, sizeof(unsigned long long))) != cudaSuccess) return bail(e, "cudaMalloc");
  if ((e = cudaMalloc(&m->scratch, sizeof(double) * 64)) != cudaSuccess) return bail(e, "cudaMalloc");
  // initial weights: uniform in +-1/sqrt(fan_in) (the output layer 10x
  // smaller, so an untrained network predicts almost no change), zero biases;
  // identity normalisation
  std::vector<float> p(kNumParams + kNumNorm, 0.f);
  uint64_t s = seed;
  auto fill = [&](int off, int out_n, int in_n, double gain) {
    const double bound = gain / std::sqrt(double(in_n));
    for (int k = 0; k < out_n * in_n; ++k) p[off + k] = float((2.0 * uniform01(s) - 1.0) * bound);
  };
  fill(kOffW1, kHid, kIn, 1.0);
  fill(kOffW2, kHid, kHid, 1.0);
  fill(kOffW3, kHid, kHid, 1.0);
  fill(kOffW4, kOut, kHid, 0.1);
  for (int k = 0; k < kIn; ++k) p[kNumParams + kNormSdX + k] = 1.f;
  for (int k = 0; k < kOut; ++k) p[kNumParams + kNormSdY + k] = 1.f;
  *out = m;
  int rc = otfem_mlp_set_state(m, p.data(), int64_t(p.size()));
  if (rc != OTFEM_OK) {
    *out = nullptr;
    otfem_mlp_destroy(m);
    return rc;
  }
  if ((e = cudaMemset(m->count, 0, sizeof(unsigned long long))) != cudaSuccess) {
    *out = nullptr;
    return bail(e, "cudaMemset");
  }
  return OTFEM_OK;
}

int otfem_mlp_destroy(otfem_mlp m) {
  if (!m) return OTFEM_OK;
  if (m->stream) cudaStreamSynchronize(m->stream);
  void* ptrs[] = {m->params, m->grad, m->adam_m, m->adam_v, m->norm, m->packed, m->X, m->Y, m->perm, m->count,
                  m->scratch};
  for (void* q : ptrs)
    if (q) cudaFree(q);
  if (m->stream) cudaStreamDestroy(m->stream);
  delete m;
  return OTFEM_OK;
}

int otfem_mlp_set_state(otfem_mlp m, const float* state, int64_t n) {
  if (!m || !state || n != OTFEM_MLP_STATE_SIZE) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  for (int k = 0; k < kIn + kOut; ++k) {
    const float sd = state[kNumParams + (k < kIn ? kNormSdX + k : kNormSdY + k - kIn)];
    if (!(sd > 0.f) || !std::isfinite(sd)) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "standard deviations must be positive");
  }
  MLP_CUDA(cudaMemcpyAsync(m->params, state, sizeof(float) * kNumParams, cudaMemcpyHostToDevice, m->stream));
  MLP_CUDA(cudaMemcpyAsync(m->norm, state + kNumParams, sizeof(float) * kNumNorm, cudaMemcpyHostToDevice, m->stream));
  MLP_CUDA(cudaMemsetAsync(m->grad, 0, sizeof(float) * kNumParams, m->stream));
  MLP_CUDA(cudaMemsetAsync(m->adam_m, 0, sizeof(float) * kNumParams, m->stream));
  MLP_CUDA(cudaMemsetAsync(m->adam_v, 0, sizeof(float) * kNumParams, m->stream));
  MLP_CUDA(cudaMemsetAsync(m->packed, 0, sizeof(__nv_bfloat16) * kPackedElems, m->stream));
  MLP_CUDA(pack(m));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  m->adam_t = 0;
  return OTFEM_OK;
}

int otfem_mlp_get_state(otfem_mlp m, float* state, int64_t n) {
  if (!m || !state || n != OTFEM_MLP_STATE_SIZE) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  MLP_CUDA(cudaMemcpyAsync(state, m->params, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaMemcpyAsync(state + kNumParams, m->norm, sizeof(float) * kNumNorm, cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return OTFEM_OK;
}

int otfem_mlp_num_samples(otfem_mlp m, int64_t* count) {
  if (!m || !count) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  unsigned long long c = 0;
  MLP_CUDA(cudaMemcpyAsync(&c, m->count, sizeof(c), cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  *count = int64_t(std::min<unsigned long long>(c, (unsigned long long)m->cap));
  return OTFEM_OK;
}

int otfem_mlp_clear_samples(otfem_mlp m) {
  if (!m) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  MLP_CUDA(cudaMemsetAsync(m->count, 0, sizeof(unsigned long long), m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return OTFEM_OK;
}

int otfem_mlp_add_samples(otfem_mlp m, otfem_handle h, double fraction, uint64_t seed, int64_t* total) {
  Context* c = context_of(h);
  if (!m || !c) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  if (!(fraction >= 0.0 && fraction <= 1.0)) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "fraction must be in [0, 1]");
  if (!c->features || !c->features_valid)
    return mlp_fail(OTFEM_ERR_NOT_INITIALIZED, "the handle's last step did not collect features (otfem_set_collect)");
  const unsigned keep = fraction >= 1.0 ? 0xffffffffu : unsigned(fraction * 4294967295.0);
  // the features and velocity changes are produced on the handle's stream
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  if (c->N > 0) {
    k_append_samples<<<(c->N + 255) / 256, 256, 0, c->stream>>>(c->N, c->fixed, c->features, c->dv_last, m->X, m->Y,
                                                                  m->count, m->cap, keep, seed);
    MLP_CUDA(cudaGetLastError());
  }
  MLP_CUDA(cudaStreamSynchronize(c->stream));
  if (total) return otfem_mlp_num_samples(m, total);
  return OTFEM_OK;
}

int otfem_mlp_fit_normalization(otfem_mlp m) {
  if (!m) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  int64_t n = 0;
  int rc = otfem_mlp_num_samples(m, &n);
  if (rc != OTFEM_OK) return rc;
  if (n < 2) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "need at least 2 samples");
  MLP_CUDA(cudaMemsetAsync(m->scratch, 0, sizeof(double) * 64, m->stream));
  k_column_moments<<<std::max(1, m->num_sms * 2), 256, 0, m->stream>>>(m->X, m->Y, n, m->scratch);
  MLP_CUDA(cudaGetLastError());
  double mom[2 * (kIn + kOut)];
  MLP_CUDA(cudaMemcpyAsync(mom, m->scratch, sizeof(mom), cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  float norm[kNumNorm];
  for (int k = 0; k < kIn + kOut; ++k) {
    const double mean = mom[k] / double(n);
    const double var = std::max(0.0, mom[kIn + kOut + k] / double(n) - mean * mean);
    double sd = std::sqrt(var);
    // an (almost) constant column: scale by its magnitude, or 1
    if (!(sd > 1e-6 * std::max(1e-30, std::fabs(mean)))) sd = std::fabs(mean) > 0.0 ? std::fabs(mean) : 1.0;
    if (k < kIn) {
      norm[kNormMuX + k] = float(mean);
      norm[kNormSdX + k] = float(sd);
    } else {
      norm[kNormMuY + k - kIn] = float(mean);
      norm[kNormSdY + k - kIn] = float(sd);
    }
  }
  MLP_CUDA(cudaMemcpyAsync(m->norm, norm, sizeof(norm), cudaMemcpyHostToDevice, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  return OTFEM_OK;
}

int otfem_mlp_train(otfem_mlp m, int32_t epochs, int32_t batch, double lr, uint64_t seed, double* last_loss) {
  if (!m || epochs < 0 || batch <= 0 || !(lr > 0.0)) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  int64_t n = 0;
  int rc = otfem_mlp_num_samples(m, &n);
  if (rc != OTFEM_OK) return rc;
  if (n == 0) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "no training samples");
  std::vector<int> perm(static_cast<size_t>(n));
  for (int64_t k = 0; k < n; ++k) perm[size_t(k)] = int(k);
  uint64_t s = seed;
  const double b1 = 0.9, b2 = 0.999, eps = 1e-8;
  double epoch_loss = 0.0;
  for (int ep = 0; ep < epochs; ++ep) {
    // Fisher-Yates shuffle
    for (int64_t k = n - 1; k > 0; --k) {
      const int64_t j = int64_t(splitmix64(s) % uint64_t(k + 1));
      std::swap(perm[size_t(k)], perm[size_t(j)]);
    }
    MLP_CUDA(cudaMemcpyAsync(m->perm, perm.data(), sizeof(int) * size_t(n), cudaMemcpyHostToDevice, m->stream));
    MLP_CUDA(cudaMemsetAsync(m->scratch, 0, sizeof(double), m->stream));
    for (int64_t off = 0; off < n; off += batch) {
      const int b = int(std::min<int64_t>(batch, n - off));
      MLP_CUDA(run_train_kernel(m, m->X, m->Y, m->perm, off, b, true));
      ++m->adam_t;
      const double c1 = 1.0 - std::pow(b1, double(m->adam_t)), c2 = 1.0 - std::pow(b2, double(m->adam_t));
      k_adam<<<(kNumParams + 255) / 256, 256, 0, m->stream>>>(m->params, m->grad, m->adam_m, m->adam_v, float(lr),
                                                              float(b1), float(b2), float(eps), float(c1), float(c2));
      MLP_CUDA(cudaGetLastError());
      MLP_CUDA(pack(m));
    }
    double sum = 0.0;
    MLP_CUDA(cudaMemcpyAsync(&sum, m->scratch, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
    MLP_CUDA(cudaStreamSynchronize(m->stream));
    epoch_loss = sum / (3.0 * double(n));
  }
  if (last_loss) *last_loss = epoch_loss;
  return OTFEM_OK;
}

int otfem_mlp_evaluate(otfem_mlp m, double* loss) {
  if (!m || !loss) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  int64_t n = 0;
  int rc = otfem_mlp_num_samples(m, &n);
  if (rc != OTFEM_OK) return rc;
  if (n == 0) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "no samples");
  std::vector<int> perm(static_cast<size_t>(n));
  for (int64_t k = 0; k < n; ++k) perm[size_t(k)] = int(k);
  MLP_CUDA(cudaMemcpyAsync(m->perm, perm.data(), sizeof(int) * size_t(n), cudaMemcpyHostToDevice, m->stream));
  MLP_CUDA(cudaMemsetAsync(m->scratch, 0, sizeof(double), m->stream));
  for (int64_t off = 0; off < n; off += (1 << 20)) {
    const int b = int(std::min<int64_t>(1 << 20, n - off));
    MLP_CUDA(run_train_kernel(m, m->X, m->Y, m->perm, off, b, false));
  }
  double sum = 0.0;
  MLP_CUDA(cudaMemcpyAsync(&sum, m->scratch, sizeof(double), cudaMemcpyDeviceToHost, m->stream));
  MLP_CUDA(cudaStreamSynchronize(m->stream));
  *loss = sum / (3.0 * double(n));
  return OTFEM_OK;
}

int otfem_mlp_gradient(otfem_mlp m, const float* x, const float* y, int64_t n, double* loss, float* grad) {
  if (!m || !x || !y || n <= 0 || n > (int64_t(1) << 30) || !loss || !grad)
    return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  float *dx = nullptr, *dy = nullptr;
  int* dp = nullptr;
  std::vector<float> hx(size_t(n) * kFeatureStride, 0.f), hy(size_t(n) * kTargetStride, 0.f);
  std::vector<int> perm(static_cast<size_t>(n));
  for (int64_t r = 0; r < n; ++r) {
    for (int k = 0; k < kIn; ++k) hx[size_t(r) * kFeatureStride + k] = x[r * kIn + k];
    for (int k = 0; k < kOut; ++k) hy[size_t(r) * kTargetStride + k] = y[r * kOut + k];
    perm[size_t(r)] = int(r);
  }
  cudaError_t e = cudaMalloc(&dx, sizeof(float) * hx.size());
  if (e == cudaSuccess) e = cudaMalloc(&dy, sizeof(float) * hy.size());
  if (e == cudaSuccess) e = cudaMalloc(&dp, sizeof(int) * perm.size());
  if (e == cudaSuccess) e = cudaMemcpyAsync(dx, hx.data(), sizeof(float) * hx.size(), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(dy, hy.data(), sizeof(float) * hy.size(), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(dp, perm.data(), sizeof(int) * perm.size(), cudaMemcpyHostToDevice, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->scratch, 0, sizeof(double), m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->grad, 0, sizeof(float) * kNumParams, m->stream);
  if (e == cudaSuccess) e = run_train_kernel(m, dx, dy, dp, 0, int(n), true);
  double sum = 0.0;
  if (e == cudaSuccess) e = cudaMemcpyAsync(&sum, m->scratch, sizeof(double), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaMemcpyAsync(grad, m->grad, sizeof(float) * kNumParams, cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(m->grad, 0, sizeof(float) * kNumParams, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  cudaFree(dx);
  cudaFree(dy);
  cudaFree(dp);
  if (e != cudaSuccess) return mlp_cuda(e, "gradient");
  *loss = sum / (3.0 * double(n));
  return OTFEM_OK;
}

int otfem_mlp_predict(otfem_mlp m, const float* x, int64_t n, float* y) {
  if (!m || !x || !y || n <= 0 || n > (int64_t(1) << 30)) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  // a one-node-per-row pseudo mesh: v, dv_prev, f_ext and the mean Re come
  // straight from x; the prediction is returned without adding dv_prev
  const int N = int(n);
  std::vector<double> v(size_t(3) * N), f(size_t(3) * N);
  std::vector<float4> d(static_cast<size_t>(N));
  std::vector<float> re(size_t(9) * N);
  std::vector<int> ptr(static_cast<size_t>(N) + 1), ent(static_cast<size_t>(N));
  for (int r = 0; r < N; ++r) {
    for (int c = 0; c < 3; ++c) {
      v[size_t(3) * r + c] = x[size_t(r) * kIn + c];
      f[size_t(3) * r + c] = x[size_t(r) * kIn + 6 + c];
    }
    d[size_t(r)] = make_float4(0.f, 0.f, 0.f, 0.f);
    for (int k = 0; k < 9; ++k) re[size_t(k) * N + r] = x[size_t(r) * kIn + 9 + k];
    ptr[size_t(r)] = r;
    ent[size_t(r)] = r << 2;
  }
  ptr[size_t(N)] = N;
  // dv_prev enters the network as an input but is not added to the output
  std::vector<float4> dprev(static_cast<size_t>(N));
  for (int r = 0; r < N; ++r)
    dprev[size_t(r)] = make_float4(x[size_t(r) * kIn + 3], x[size_t(r) * kIn + 4], x[size_t(r) * kIn + 5], 0.f);
  Context c;
  c.N = N;
  c.T = N;
  c.stream = m->stream;
  c.mlp = m;
  std::vector<unsigned char> fixed(static_cast<size_t>(N), 0);
  cudaError_t e = cudaSuccess;
  void* bufs[8] = {nullptr};
  auto alloc = [&](void** p, size_t bytes, const void* src) {
    if (e != cudaSuccess) return;
    e = cudaMalloc(p, bytes);
    if (e == cudaSuccess && src) e = cudaMemcpyAsync(*p, src, bytes, cudaMemcpyHostToDevice, m->stream);
  };
  alloc(&bufs[0], sizeof(double) * v.size(), v.data());
  alloc(&bufs[1], sizeof(double) * f.size(), f.data());
  alloc(&bufs[2], sizeof(float4) * dprev.size(), dprev.data());
  alloc(&bufs[3], sizeof(float) * re.size(), re.data());
  alloc(&bufs[4], sizeof(int) * ptr.size(), ptr.data());
  alloc(&bufs[5], sizeof(int) * ent.size(), ent.data());
  alloc(&bufs[6], fixed.size(), fixed.data());
  alloc(&bufs[7], sizeof(float4) * size_t(N), nullptr);
  if (e == cudaSuccess) {
    c.v = static_cast<double*>(bufs[0]);
    c.fext = static_cast<double*>(bufs[1]);
    c.dv_last = static_cast<float4*>(bufs[2]);
    c.re_f = static_cast<float*>(bufs[3]);
    c.inc_ptr = static_cast<int*>(bufs[4]);
    c.inc_ent = static_cast<int*>(bufs[5]);
    c.fixed = static_cast<unsigned char*>(bufs[6]);
    c.warm_dv = static_cast<float4*>(bufs[7]);
    e = launch_node_features(c, true);
  }
  std::vector<float4> out(static_cast<size_t>(N));
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(out.data(), bufs[7], sizeof(float4) * size_t(N), cudaMemcpyDeviceToHost, m->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(m->stream);
  for (void* b : bufs)
    if (b) cudaFree(b);
  // the pseudo mesh must not free the buffers it borrowed
  c.v = nullptr, c.fext = nullptr, c.dv_last = nullptr, c.re_f = nullptr, c.inc_ptr = nullptr, c.inc_ent = nullptr;
  c.fixed = nullptr, c.warm_dv = nullptr, c.stream = nullptr, c.mlp = nullptr;
  if (e != cudaSuccess) return mlp_cuda(e, "predict");
  for (int r = 0; r < N; ++r) {
    y[size_t(r) * kOut + 0] = out[size_t(r)].x - dprev[size_t(r)].x;
    y[size_t(r) * kOut + 1] = out[size_t(r)].y - dprev[size_t(r)].y;
    y[size_t(r) * kOut + 2] = out[size_t(r)].z - dprev[size_t(r)].z;
  }
  return OTFEM_OK;
}

int otfem_set_mlp(otfem_handle h, otfem_mlp m) {
  Context* c = context_of(h);
  if (!c) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  // kernel attributes outside any stream capture of the step
  if (cudaError_t e = set_attributes()) return mlp_cuda(e, "cudaFuncSetAttribute");
  if (m && m->device != c->device) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "network and mesh on different devices");
  if (m && !c->warm_tmp) {
    cudaError_t e = cudaMalloc(&c->warm_tmp, sizeof(float4) * size_t(std::max(c->N, 1)));
    if (e != cudaSuccess) return mlp_cuda(e, "cudaMalloc");
  }
  c->mlp = m;
  return OTFEM_OK;
}

int otfem_get_features(otfem_handle h, float* out, int64_t n) {
  Context* c = context_of(h);
  if (!c || !out) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "null argument");
  if (n != int64_t(kFeatures) * c->N) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "n must be 18 * num_nodes");
  if (!c->features || !c->features_valid)
    return mlp_fail(OTFEM_ERR_NOT_INITIALIZED, "the last step did not collect features (otfem_set_collect)");
  std::vector<float> buf(size_t(kFeatureStride) * size_t(c->N));
  cudaError_t e = cudaMemcpyAsync(buf.data(), c->features, sizeof(float) * buf.size(), cudaMemcpyDeviceToHost,
                                  c->stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
  if (e != cudaSuccess) return mlp_cuda(e, "features");
  for (int i = 0; i < c->N; ++i)
    for (int k = 0; k < kFeatures; ++k) out[size_t(i) * kFeatures + k] = buf[size_t(i) * kFeatureStride + k];
  return OTFEM_OK;
}

int otfem_set_warm_start_smoothing(otfem_handle h, int32_t passes) {
  Context* c = context_of(h);
  if (!c || passes < 0 || passes > 64) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "bad argument");
  if (passes > 0 && !c->warm_tmp) {
    cudaError_t e = cudaMalloc(&c->warm_tmp, sizeof(float4) * size_t(std::max(c->N, 1)));
    if (e != cudaSuccess) return mlp_cuda(e, "cudaMalloc");
  }
  c->warm_smoothing = passes;
  drop_step_graphs(*c);
  return OTFEM_OK;
}

int otfem_set_collect(otfem_handle h, int32_t enable) {
  Context* c = context_of(h);
  if (!c) return mlp_fail(OTFEM_ERR_INVALID_ARGUMENT, "null handle");
  if (cudaError_t e = set_attributes()) return mlp_cuda(e, "cudaFuncSetAttribute");
  if (enable && !c->features) {
    cudaError_t e = cudaMalloc(&c->features, sizeof(float) * kFeatureStride * size_t(std::max(c->N, 1)));
    if (e != cudaSuccess) return mlp_cuda(e, "cudaMalloc features");
  }
  c->collect = enable ? 1 : 0;
  c->features_valid = false;
  return OTFEM_OK;
}

}  // extern "C"
