// ace_mlp.cu -- the learned radial form: an MLP that maps (r, neighbour
// species) to K radial channels per l, evaluated per neighbour ahead of the
// energy/force kernel, its backward pass and an Adam step for training it.
//
// Model (per neighbour j at distance r with species s):
//   t = ((1 + r0) / (1 + r))^p            the basis' own distance transform
//   fe(t) = (t - tl)^pl (t - tr)^pr       its cutoff envelope (0 outside)
//   x = 2 (t - tl) / (tmax - tl) - 1      features T_0..T_{Q-1}(x) (Chebyshev)
//   f = [T_0(x) .. T_{Q-1}(x), onehot(s)] (D = Q + S inputs)
//   h1 = silu(W1 f + b1), h2 = silu(W2 h1 + b2)   (H = 64 each)
//   o = W3 h2 + b3                        (C = K (L+1) outputs)
//   R_c(r, s) = fe(t) o_c                 channel c = k + K l
// dR_c/dr follows by forward-mode differentiation in t.  Parameters are one
// FP32 array [W1 (H x D) | b1 | W2 (H x H) | b2 | W3 (C x H) | b3].
//
// This form is not in ACE.jl: it compresses the species- and degree-resolved
// radial basis R_n(r) x species of src/b1pcomponents/Rn.jl and
// src/discrete1pbasis.jl into K learned channels per l.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <string>
#include <vector>

#include <cuda_bf16.h>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_phi.cuh"

namespace ace {

constexpr int MLP_H = 64;
constexpr int MLP_MAXQ = 16;
constexpr int MLP_MAXS = 8;
constexpr int MLP_MAXD = MLP_MAXQ + MLP_MAXS;
constexpr int MLP_MAXC = 512;
constexpr int NTF = 128;  // forward: neighbours per CTA
constexpr int NTB = 64;   // backward: neighbours per CTA
constexpr int PSB = NTB + 1;

struct MLPOff {
  int64_t W1, b1, W2, b2, W3, b3, n;
};

__host__ __device__ inline MLPOff mlp_off(int H, int D, int C) {
  MLPOff o;
  o.W1 = 0;
  o.b1 = o.W1 + (int64_t)H * D;
  o.W2 = o.b1 + H;
  o.b2 = o.W2 + (int64_t)H * H;
  o.W3 = o.b2 + H;
  o.b3 = o.W3 + (int64_t)C * H;
  o.n = o.b3 + C;
  return o;
}

struct MLPArgs {
  int64_t n;              // neighbours; < 0: off[nEnv]
  const int64_t *off;
  int64_t nEnv;
  const double *rr;
  const int32_t *sp;
  const float *W;
  int D, Q, S, C;
  float a0, tl, tr, xs;   // 1 + r0, envelope roots, feature scale 2 / (tmax - tl)
  int tp, pl, pr;
  float *R;               // forward: [n][2C] (R, then dR/dr)
  const float *gR;        // backward: dL/dR [n][C]
  const float *wj;        // backward: per-neighbour weight (NULL = 1)
  float *gW;              // backward: accumulated parameter gradient
  int *status;
  int64_t wait_limit;     // tensor-core kernel: polls of an MMA completion before giving up
};

struct Feat {
  float dtdr, fe, dfe;
};

__device__ __forceinline__ float ipowf(float x, int p) {
  float r = 1.f;
  for (int i = 0; i < p; ++i) r *= x;
  return r;
}

// transform, envelope and features of neighbour j; df = d f / dt (first Q)
__device__ __forceinline__ Feat mlp_inputs(const MLPArgs &a, int64_t j, float (&f)[MLP_MAXD],
                                           float (&df)[MLP_MAXQ]) {
  const double xd = a.rr[3 * j], yd = a.rr[3 * j + 1], zd = a.rr[3 * j + 2];
  const float r = (float)sqrt(xd * xd + yd * yd + zd * zd);
  const float u = 1.f + r;
  const float x = a.a0 / u;
  const float t = ipowf(x, a.tp);
  Feat q;
  q.dtdr = (float)a.tp * ipowf(x, a.tp - 1) * (-(a.a0 / (u * u)));
  const bool outside = (a.pl > 0 && t < a.tl) || (a.pr > 0 && t > a.tr);
  q.fe = outside ? 0.f : ipowf(t - a.tl, a.pl) * ipowf(t - a.tr, a.pr);
  q.dfe = 0.f;
  if (!outside) {
    if (a.pl > 0) q.dfe += (float)a.pl * ipowf(t - a.tl, a.pl - 1) * ipowf(t - a.tr, a.pr);
    if (a.pr > 0) q.dfe += ipowf(t - a.tl, a.pl) * (float)a.pr * ipowf(t - a.tr, a.pr - 1);
  }
  const float z = a.xs * (t - a.tl) - 1.f;
  // Chebyshev T_q(z) and dT_q/dz by the three-term recurrence
  float T0 = 1.f, T1 = z, d0 = 0.f, d1 = 1.f;
#pragma unroll
  for (int k = 0; k < MLP_MAXQ; ++k) {
    float Tk, dk;
    if (k == 0) { Tk = T0; dk = d0; }
    else if (k == 1) { Tk = T1; dk = d1; }
    else {
      Tk = 2.f * z * T1 - T0;
      dk = 2.f * T1 + 2.f * z * d1 - d0;
      T0 = T1; T1 = Tk; d0 = d1; d1 = dk;
    }
    if (k < a.Q) { f[k] = Tk; df[k] = dk * a.xs; }
  }
  int s = a.sp ? a.sp[j] : 0;
  if (s < 0 || s >= a.S) {
    atomicOr(a.status, ACE_STATUS_BAD_SPECIES);
    s = 0;
  }
#pragma unroll
  for (int d = 0; d < MLP_MAXD; ++d)
    if (d >= a.Q && d < a.Q + a.S) f[d] = (d - a.Q == s) ? 1.f : 0.f;
  return q;
}

__device__ __forceinline__ float sigm(float z) { return 1.f / (1.f + expf(-z)); }

// parameters into shared memory, W2 transposed (W2T[k][i] = W2[i][k])
__device__ __forceinline__ void load_params(const MLPArgs &a, const MLPOff &o, float *W) {
  for (int64_t i = threadIdx.x; i < o.n; i += blockDim.x) {
    float v = a.W[i];
    int64_t d = i;
    if (i >= o.W2 && i < o.b2) {
      const int64_t q = i - o.W2, r = q / MLP_H, c = q - r * MLP_H;
      d = o.W2 + c * MLP_H + r;
    }
    W[d] = v;
  }
}

// forward: one thread per neighbour; h1 and its t-tangent in shared memory,
// h2 in registers, outputs one channel at a time
__global__ void __launch_bounds__(NTF) mlp_fwd_kernel(MLPArgs a) {
  constexpr int H = MLP_H;
  extern __shared__ __align__(16) float smf[];
  const MLPOff o = mlp_off(H, a.D, a.C);
  float *W = smf;
  float *h1 = smf + ((o.n + 3) & ~int64_t(3));
  float *dh1 = h1 + H * NTF;
  load_params(a, o, W);
  __syncthreads();
  const int64_t n = a.n >= 0 ? a.n : a.off[a.nEnv];
  const int tid = threadIdx.x;
  for (int64_t base = (int64_t)blockIdx.x * NTF; base < n; base += (int64_t)gridDim.x * NTF) {
    const int64_t j = base + tid;
    const bool act = j < n;
    float f[MLP_MAXD], df[MLP_MAXQ];
    const Feat q = mlp_inputs(a, act ? j : n - 1, f, df);
    for (int i = 0; i < H; ++i) {
      float z = W[o.b1 + i], dz = 0.f;
      const float *w1 = W + o.W1 + i * a.D;
#pragma unroll
      for (int d = 0; d < MLP_MAXD; ++d)
        if (d < a.D) z = fmaf(w1[d], f[d], z);
#pragma unroll
      for (int d = 0; d < MLP_MAXQ; ++d)
        if (d < a.Q) dz = fmaf(w1[d], df[d], dz);
      const float sg = sigm(z);
      h1[i * NTF + tid] = z * sg;
      dh1[i * NTF + tid] = sg * (1.f + z * (1.f - sg)) * dz;
    }
    float z2[H], d2[H];
#pragma unroll
    for (int i = 0; i < H; ++i) { z2[i] = W[o.b2 + i]; d2[i] = 0.f; }
    for (int k = 0; k < H; ++k) {
      const float hk = h1[k * NTF + tid], dk = dh1[k * NTF + tid];
      const float4 *w = (const float4 *)(W + o.W2 + k * H);
#pragma unroll
      for (int i4 = 0; i4 < H / 4; ++i4) {
        const float4 v = w[i4];
        z2[4 * i4 + 0] = fmaf(v.x, hk, z2[4 * i4 + 0]); d2[4 * i4 + 0] = fmaf(v.x, dk, d2[4 * i4 + 0]);
        z2[4 * i4 + 1] = fmaf(v.y, hk, z2[4 * i4 + 1]); d2[4 * i4 + 1] = fmaf(v.y, dk, d2[4 * i4 + 1]);
        z2[4 * i4 + 2] = fmaf(v.z, hk, z2[4 * i4 + 2]); d2[4 * i4 + 2] = fmaf(v.z, dk, d2[4 * i4 + 2]);
        z2[4 * i4 + 3] = fmaf(v.w, hk, z2[4 * i4 + 3]); d2[4 * i4 + 3] = fmaf(v.w, dk, d2[4 * i4 + 3]);
      }
    }
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const float sg = sigm(z2[i]);
      d2[i] = sg * (1.f + z2[i] * (1.f - sg)) * d2[i];
      z2[i] = z2[i] * sg;
    }
    for (int c = 0; c < a.C; ++c) {
      const float4 *w = (const float4 *)(W + o.W3 + (int64_t)c * H);
      float ov = W[o.b3 + c], dv = 0.f;
#pragma unroll
      for (int i4 = 0; i4 < H / 4; ++i4) {
        const float4 v = w[i4];
        ov = fmaf(v.x, z2[4 * i4 + 0], ov); dv = fmaf(v.x, d2[4 * i4 + 0], dv);
        ov = fmaf(v.y, z2[4 * i4 + 1], ov); dv = fmaf(v.y, d2[4 * i4 + 1], dv);
        ov = fmaf(v.z, z2[4 * i4 + 2], ov); dv = fmaf(v.z, d2[4 * i4 + 2], dv);
        ov = fmaf(v.w, z2[4 * i4 + 3], ov); dv = fmaf(v.w, d2[4 * i4 + 3], dv);
      }
      if (act) {
        a.R[(size_t)j * 2 * a.C + c] = q.fe * ov;
        a.R[(size_t)j * 2 * a.C + a.C + c] = (q.dfe * ov + q.fe * dv) * q.dtdr;
      }
    }
  }
}

// backward: dL/dparams += sum_j wj dL/dR_j . dR_j/dparams (values only).
// One thread per neighbour for the per-neighbour vectors; the outer-product
// reductions over the tile's neighbours are done from shared memory with each
// parameter owned by one thread, accumulated over the CTA's tiles in shared
// memory and added to gW once per CTA.
__global__ void __launch_bounds__(NTB) mlp_bwd_kernel(MLPArgs a) {
  constexpr int H = MLP_H;
  extern __shared__ __align__(16) float smf[];
  const MLPOff o = mlp_off(H, a.D, a.C);
  const int64_t npa = (o.n + 3) & ~int64_t(3);
  float *W = smf;
  float *gacc = W + npa;
  float *h1 = gacc + npa;          // [H][PSB]
  float *s1 = h1 + H * PSB;        // silu'(z1), later dL/dz1
  float *h2s = s1 + H * PSB;       // [H][PSB]
  float *fs = h2s + H * PSB;       // [D][PSB]
  float *stg = fs + MLP_MAXD * PSB;  // [max(C, H)][PSB]: dL/do, later dL/dz2
  load_params(a, o, W);
  for (int64_t i = threadIdx.x; i < o.n; i += NTB) gacc[i] = 0.f;
  __syncthreads();
  const int64_t n = a.n >= 0 ? a.n : a.off[a.nEnv];
  const int tid = threadIdx.x;
  for (int64_t base = (int64_t)blockIdx.x * NTB; base < n; base += (int64_t)gridDim.x * NTB) {
    const int64_t j = base + tid;
    const bool act = j < n;
    const int64_t jc = act ? j : n - 1;
    float f[MLP_MAXD], df[MLP_MAXQ];
    const Feat q = mlp_inputs(a, jc, f, df);
#pragma unroll
    for (int d = 0; d < MLP_MAXD; ++d)
      if (d < a.D) fs[d * PSB + tid] = f[d];
    for (int i = 0; i < H; ++i) {
      float z = W[o.b1 + i];
      const float *w1 = W + o.W1 + i * a.D;
#pragma unroll
      for (int d = 0; d < MLP_MAXD; ++d)
        if (d < a.D) z = fmaf(w1[d], f[d], z);
      const float sg = sigm(z);
      h1[i * PSB + tid] = z * sg;
      s1[i * PSB + tid] = sg * (1.f + z * (1.f - sg));
    }
    float z2[H];
#pragma unroll
    for (int i = 0; i < H; ++i) z2[i] = W[o.b2 + i];
    for (int k = 0; k < H; ++k) {
      const float hk = h1[k * PSB + tid];
      const float4 *w = (const float4 *)(W + o.W2 + k * H);
#pragma unroll
      for (int i4 = 0; i4 < H / 4; ++i4) {
        const float4 v = w[i4];
        z2[4 * i4 + 0] = fmaf(v.x, hk, z2[4 * i4 + 0]);
        z2[4 * i4 + 1] = fmaf(v.y, hk, z2[4 * i4 + 1]);
        z2[4 * i4 + 2] = fmaf(v.z, hk, z2[4 * i4 + 2]);
        z2[4 * i4 + 3] = fmaf(v.w, hk, z2[4 * i4 + 3]);
      }
    }
    float s2[H];
#pragma unroll
    for (int i = 0; i < H; ++i) {
      const float sg = sigm(z2[i]);
      s2[i] = sg * (1.f + z2[i] * (1.f - sg));
      h2s[i * PSB + tid] = z2[i] * sg;
    }
    const float sc = act ? q.fe * (a.wj ? a.wj[j] : 1.f) : 0.f;
    for (int c = 0; c < a.C; ++c) stg[c * PSB + tid] = act ? a.gR[(size_t)j * a.C + c] * sc : 0.f;
    __syncthreads();
    // W3, b3
    for (int64_t idx = tid; idx < (int64_t)a.C * (H + 1); idx += NTB) {
      const int c = (int)(idx / (H + 1)), i = (int)(idx - (int64_t)c * (H + 1));
      const float *g = stg + c * PSB;
      float acc = 0.f;
      if (i < H) {
        const float *h = h2s + i * PSB;
        for (int t = 0; t < NTB; ++t) acc = fmaf(g[t], h[t], acc);
        gacc[o.W3 + (int64_t)c * H + i] += acc;
      } else {
        for (int t = 0; t < NTB; ++t) acc += g[t];
        gacc[o.b3 + c] += acc;
      }
    }
    // dL/dz2 = s2 * W3^T dL/do (per thread)
    float g2[H];
#pragma unroll
    for (int i = 0; i < H; ++i) g2[i] = 0.f;
    for (int c = 0; c < a.C; ++c) {
      const float g = stg[c * PSB + tid];
      const float4 *w = (const float4 *)(W + o.W3 + (int64_t)c * H);
#pragma unroll
      for (int i4 = 0; i4 < H / 4; ++i4) {
        const float4 v = w[i4];
        g2[4 * i4 + 0] = fmaf(v.x, g, g2[4 * i4 + 0]);
        g2[4 * i4 + 1] = fmaf(v.y, g, g2[4 * i4 + 1]);
        g2[4 * i4 + 2] = fmaf(v.z, g, g2[4 * i4 + 2]);
        g2[4 * i4 + 3] = fmaf(v.w, g, g2[4 * i4 + 3]);
      }
    }
    __syncthreads();
#pragma unroll
    for (int i = 0; i < H; ++i) {
      g2[i] *= s2[i];
      stg[i * PSB + tid] = g2[i];
    }
    __syncthreads();
    // W2, b2 (parameter layout W2[i][k])
    for (int64_t idx = tid; idx < (int64_t)H * (H + 1); idx += NTB) {
      const int i = (int)(idx / (H + 1)), k = (int)(idx - (int64_t)i * (H + 1));
      const float *g = stg + i * PSB;
      float acc = 0.f;
      if (k < H) {
        const float *h = h1 + k * PSB;
        for (int t = 0; t < NTB; ++t) acc = fmaf(g[t], h[t], acc);
        gacc[o.W2 + (int64_t)i * H + k] += acc;
      } else {
        for (int t = 0; t < NTB; ++t) acc += g[t];
        gacc[o.b2 + i] += acc;
      }
    }
    // dL/dz1 = s1 * W2^T dL/dz2 (per thread, into s1)
    for (int k = 0; k < H; ++k) {
      const float4 *w = (const float4 *)(W + o.W2 + k * H);  // W2T[k][*] = W2[*][k]
      float acc = 0.f;
#pragma unroll
      for (int i4 = 0; i4 < H / 4; ++i4) {
        const float4 v = w[i4];
        acc = fmaf(v.x, g2[4 * i4 + 0], acc);
        acc = fmaf(v.y, g2[4 * i4 + 1], acc);
        acc = fmaf(v.z, g2[4 * i4 + 2], acc);
        acc = fmaf(v.w, g2[4 * i4 + 3], acc);
      }
      s1[k * PSB + tid] *= acc;
    }
    __syncthreads();
    // W1, b1
    for (int64_t idx = tid; idx < (int64_t)H * (a.D + 1); idx += NTB) {
      const int i = (int)(idx / (a.D + 1)), d = (int)(idx - (int64_t)i * (a.D + 1));
      const float *g = s1 + i * PSB;
      float acc = 0.f;
      if (d < a.D) {
        const float *x = fs + d * PSB;
        for (int t = 0; t < NTB; ++t) acc = fmaf(g[t], x[t], acc);
        gacc[o.W1 + (int64_t)i * a.D + d] += acc;
      } else {
        for (int t = 0; t < NTB; ++t) acc += g[t];
        gacc[o.b1 + i] += acc;
      }
    }
    __syncthreads();
  }
  for (int64_t i = tid; i < o.n; i += NTB) atomicAdd(a.gW + i, gacc[i]);
}

__global__ void adam_kernel(int64_t n, float *w, const float *g, float *m, float *v, float lr, float b1, float b2,
                            float eps, float bc1, float bc2) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    w[i] -= lr * (mi / bc1) / (sqrtf(vi / bc2) + eps);
  }
}

// ---------------------------------------------------------------------------
// Tensor-core inference: the same MLP with BF16 operands and FP32
// accumulation on the 5th-generation tensor cores.  One CTA (4 warps) takes
// 128 neighbours at a time; each layer is two tcgen05.mma GEMMs (values and
// their t-tangents) of M = 128 rows against the layer's weights, issued by one
// thread from shared memory into TMEM, completion signalled through an
// mbarrier; the epilogue reads each thread's row back with tcgen05.ld, applies
// bias and SiLU (and the tangent chain rule) in FP32 and stores the next
// layer's BF16 operand.  Operands use the no-swizzle K-major layout: 8-row x
// 16-byte core matrices, LBO = 128 B between core matrices along K, SBO =
// K * 16 B between 8-row groups.

constexpr uint32_t TC_COLS = 256;        // TMEM columns per CTA: values at 0, tangents at 128
constexpr int TC_N3 = 128;               // output channels padded to a multiple of 16 (K (L+1) <= 128)
constexpr int TC_K1 = 16;                // layer-1 inputs padded to one MMA K step

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start, leading and stride byte offsets,
// fixed version bits 46-48 = 0b001, no swizzle
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
         ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | (1ull << 46);
}

// instruction descriptor, kind::f16: FP32 accumulator, BF16 A and B, both K-major
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void umma_bf16(uint32_t dtmem, uint64_t ad, uint64_t bd, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}\n" ::"r"(dtmem),
      "l"(ad), "l"(bd), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void umma_commit(uint32_t mbar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(mbar)
               : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool mbar_wait(uint32_t mbar, uint32_t parity, int64_t limit) {
  for (int64_t i = 0; i < limit; ++i) {
    uint32_t done;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}\n"
        : "=r"(done)
        : "r"(mbar), "r"(parity)
        : "memory");
    if (done) return true;
  }
  return false;
}

// 16 consecutive FP32 columns of this warp's 32 TMEM lanes (one row per thread)
__device__ __forceinline__ void tmem_ld16(uint32_t taddr, float (&v)[16]) {
  uint32_t r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; ++i) v[i] = __uint_as_float(r[i]);
}

// byte offset of element (row, k) in a K-major no-swizzle operand with K columns
__device__ __forceinline__ uint32_t kmaj_off(int row, int k, int K) {
  return (uint32_t)((row >> 3) * (K * 16) + (k >> 3) * 128 + (row & 7) * 16 + (k & 7) * 2);
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *(const uint32_t *)&v;
}

// 8 consecutive k of one row (one core-matrix row, 16 bytes)
__device__ __forceinline__ void st_row8(unsigned char *base, int row, int k0, int K, const float *x) {
  uint4 q;
  q.x = pack_bf16(x[0], x[1]);
  q.y = pack_bf16(x[2], x[3]);
  q.z = pack_bf16(x[4], x[5]);
  q.w = pack_bf16(x[6], x[7]);
  *(uint4 *)(base + kmaj_off(row, k0, K)) = q;
}

struct TCSmem {
  // operands (BF16, K-major core-matrix layout)
  unsigned char W1[MLP_H * TC_K1 * 2];
  unsigned char W2[MLP_H * MLP_H * 2];
  unsigned char W3[TC_N3 * MLP_H * 2];
  unsigned char X[2][128 * MLP_H * 2];   // [0] F / H2 values, [1] their tangents
  unsigned char Y[2][128 * MLP_H * 2];   // H1 values, tangents
  float b1[MLP_H], b2[MLP_H], b3[TC_N3];
  unsigned long long mbar;
  uint32_t taddr;
};

__global__ void __launch_bounds__(128) mlp_fwd_tc_kernel(MLPArgs a) {
  constexpr int H = MLP_H;
  extern __shared__ __align__(1024) unsigned char smraw[];
  TCSmem &S = *(TCSmem *)smraw;
  const int tid = threadIdx.x, warp = tid >> 5;
  const MLPOff o = mlp_off(H, a.D, a.C);
  // weights -> BF16 operands (zero padding), biases -> FP32
  for (int i = tid; i < H * TC_K1; i += 128) {
    const int n = i / TC_K1, k = i - n * TC_K1;
    const float w = (k < a.D) ? a.W[o.W1 + n * a.D + k] : 0.f;
    *(__nv_bfloat16 *)(S.W1 + kmaj_off(n, k, TC_K1)) = __float2bfloat16_rn(w);
  }
  for (int i = tid; i < H * H; i += 128) {
    const int n = i / H, k = i - n * H;
    *(__nv_bfloat16 *)(S.W2 + kmaj_off(n, k, H)) = __float2bfloat16_rn(a.W[o.W2 + i]);
  }
  for (int i = tid; i < TC_N3 * H; i += 128) {
    const int n = i / H, k = i - n * H;
    const float w = (n < a.C) ? a.W[o.W3 + (int64_t)n * H + k] : 0.f;
    *(__nv_bfloat16 *)(S.W3 + kmaj_off(n, k, H)) = __float2bfloat16_rn(w);
  }
  for (int i = tid; i < H; i += 128) { S.b1[i] = a.W[o.b1 + i]; S.b2[i] = a.W[o.b2 + i]; }
  for (int i = tid; i < TC_N3; i += 128) S.b3[i] = (i < a.C) ? a.W[o.b3 + i] : 0.f;
  const uint32_t mbar = smem_u32(&S.mbar);
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&S.taddr)),
                 "r"(TC_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  fence_async_smem();
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = S.taddr;
  const uint32_t trow = tmem + ((uint32_t)(32 * warp) << 16);  // this warp's lanes
  const uint32_t i1 = umma_idesc(128, H), i3 = umma_idesc(128, TC_N3);
  const int64_t limit = int64_t(1) << 26;
  uint32_t phase = 0;
  bool ok = true;
  const int64_t n = a.n >= 0 ? a.n : a.off[a.nEnv];

  // one layer: D_values = X[0] W^T, D_tangents = X[1] W^T over nk K-steps of 16
  auto issue = [&](unsigned char *const *A, const unsigned char *W, int K, int nk, uint32_t idesc) {
    fence_async_smem();
    tc_fence_before();
    __syncthreads();
    if (tid == 0) {
      tc_fence_after();
      for (int v = 0; v < 2; ++v)
        for (int s = 0; s < nk; ++s)
          umma_bf16(tmem + (uint32_t)(128 * v), umma_desc(smem_u32(A[v]) + 256u * s, 128u, (uint32_t)(K * 16)),
                    umma_desc(smem_u32(W) + 256u * s, 128u, (uint32_t)(K * 16)), idesc, s > 0 ? 1u : 0u);
      umma_commit(mbar);
    }
    // a wait that gives up leaves the phase pending (waited on again before
    // the TMEM is freed); the block agrees on the outcome
    const bool done = __syncthreads_and(mbar_wait(mbar, phase, a.wait_limit) ? 1 : 0) != 0;
    if (done) phase ^= 1u;
    tc_fence_after();
    return done;
  };

  for (int64_t base = (int64_t)blockIdx.x * 128; base < n && ok; base += (int64_t)gridDim.x * 128) {
    const int64_t j = base + tid;
    const bool act = j < n;
    float f[MLP_MAXD], df[MLP_MAXQ];
    const Feat q = mlp_inputs(a, act ? j : n - 1, f, df);
    {
      float x[16], dx[16];
#pragma unroll
      for (int k = 0; k < 16; ++k) {
        x[k] = (k < a.D) ? f[k < MLP_MAXD ? k : 0] : 0.f;
        dx[k] = (k < a.Q) ? df[k < MLP_MAXQ ? k : 0] : 0.f;
      }
      st_row8(S.X[0], tid, 0, TC_K1, x);
      st_row8(S.X[0], tid, 8, TC_K1, x + 8);
      st_row8(S.X[1], tid, 0, TC_K1, dx);
      st_row8(S.X[1], tid, 8, TC_K1, dx + 8);
    }
    unsigned char *X[2] = {S.X[0], S.X[1]};
    unsigned char *Y[2] = {S.Y[0], S.Y[1]};
    if (!issue(X, S.W1, TC_K1, 1, i1)) { ok = false; break; }
    // layer-1 epilogue -> Y
#pragma unroll
    for (int c0 = 0; c0 < H; c0 += 16) {
      float z[16], dz[16], h[16], dh[16];
      tmem_ld16(trow + c0, z);
      tmem_ld16(trow + 128 + c0, dz);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const float zz = z[i] + S.b1[c0 + i];
        const float sg = sigm(zz);
        h[i] = zz * sg;
        dh[i] = sg * (1.f + zz * (1.f - sg)) * dz[i];
      }
      st_row8(Y[0], tid, c0, H, h);
      st_row8(Y[0], tid, c0 + 8, H, h + 8);
      st_row8(Y[1], tid, c0, H, dh);
      st_row8(Y[1], tid, c0 + 8, H, dh + 8);
    }
    if (!issue(Y, S.W2, H, H / 16, i1)) { ok = false; break; }
    // layer-2 epilogue -> X
#pragma unroll
    for (int c0 = 0; c0 < H; c0 += 16) {
      float z[16], dz[16], h[16], dh[16];
      tmem_ld16(trow + c0, z);
      tmem_ld16(trow + 128 + c0, dz);
#pragma unroll
      for (int i = 0; i < 16; ++i) {
        const float zz = z[i] + S.b2[c0 + i];
        const float sg = sigm(zz);
        h[i] = zz * sg;
        dh[i] = sg * (1.f + zz * (1.f - sg)) * dz[i];
      }
      st_row8(X[0], tid, c0, H, h);
      st_row8(X[0], tid, c0 + 8, H, h + 8);
      st_row8(X[1], tid, c0, H, dh);
      st_row8(X[1], tid, c0 + 8, H, dh + 8);
    }
    if (!issue(X, S.W3, H, H / 16, i3)) { ok = false; break; }
    // output epilogue: 32 channels at a time staged in the (free) H1 buffers
    // as [row][R 32 | dR 32] and stored row segment by row segment, 16 bytes
    // per thread, so a warp writes whole 128-byte lines
    float *stage = (float *)S.Y[0];
    const int nrow = (n - base < 128) ? (int)(n - base) : 128;
    for (int c0 = 0; c0 < TC_N3; c0 += 32) {
      float ov[32], dv[32];
      tmem_ld16(trow + c0, *(float(*)[16])ov);
      tmem_ld16(trow + c0 + 16, *(float(*)[16])(ov + 16));
      tmem_ld16(trow + 128 + c0, *(float(*)[16])dv);
      tmem_ld16(trow + 128 + c0 + 16, *(float(*)[16])(dv + 16));
#pragma unroll
      for (int i = 0; i < 32; ++i) {
        const int c = c0 + i;
        const float y = ov[i] + S.b3[c < TC_N3 ? c : 0];
        // row-rotated columns keep the staging writes conflict free
        stage[tid * 64 + ((i + tid) & 31)] = q.fe * y;
        stage[tid * 64 + 32 + ((i + tid) & 31)] = (q.dfe * y + q.fe * dv[i]) * q.dtdr;
      }
      __syncthreads();
      const int nc = (a.C - c0 < 32) ? a.C - c0 : 32;  // channels of this chunk (a multiple of 4)
      const int per_row = 2 * (nc / 4);       // float4 pieces of a row: R then dR
      for (int p = tid; p < nrow * per_row; p += 128) {
        const int r = p / per_row, w = p - r * per_row;
        const int half = w >= nc / 4, c4 = (half ? w - nc / 4 : w) * 4;
        float4 v;
        const float *src = stage + r * 64 + half * 32;
        v.x = src[(c4 + 0 + r) & 31];
        v.y = src[(c4 + 1 + r) & 31];
        v.z = src[(c4 + 2 + r) & 31];
        v.w = src[(c4 + 3 + r) & 31];
        *(float4 *)(a.R + (size_t)(base + r) * 2 * a.C + half * a.C + c0 + c4) = v;
      }
      __syncthreads();
    }
  }
  if (!ok) {
    // the MMAs still in flight complete before their TMEM is freed (bounded
    // by the full limit even when a shorter one was given for the waits above)
    if (tid == 0) atomicOr(a.status, ACE_STATUS_TIMEOUT);
    mbar_wait(mbar, phase, limit);
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TC_COLS) : "memory");
}

static MLPArgs mlp_args(const ace_ctx *ctx) {
  MLPArgs a{};
  a.W = ctx->d_mlp;
  a.D = ctx->mlpD; a.Q = ctx->mlpQ; a.S = ctx->mlpS; a.C = ctx->mlpC;
  a.a0 = (float)(1.0 + ctx->r0);
  a.tl = (float)ctx->tl; a.tr = (float)ctx->tr;
  a.xs = (float)(2.0 / (ctx->mlp_tmax - ctx->tl));
  a.tp = ctx->tp; a.pl = ctx->pl; a.pr = ctx->pr;
  a.status = ctx->d_status;
  a.wait_limit = ctx->tc_wait_limit;
  return a;
}

static size_t fwd_smem(const ace_ctx *ctx) {
  const MLPOff o = mlp_off(MLP_H, ctx->mlpD, ctx->mlpC);
  return (size_t)(((o.n + 3) & ~int64_t(3)) + 2 * MLP_H * NTF) * sizeof(float);
}

static size_t bwd_smem(const ace_ctx *ctx) {
  const MLPOff o = mlp_off(MLP_H, ctx->mlpD, ctx->mlpC);
  const int64_t npa = (o.n + 3) & ~int64_t(3);
  return (size_t)(2 * npa + (3 * MLP_H + MLP_MAXD + std::max(ctx->mlpC, MLP_H)) * PSB) * sizeof(float);
}

int mlp_prepare(ace_ctx *ctx) {
  // polls of a tensor-core completion before the kernel gives up and sets
  // ACE_STATUS_TIMEOUT; ACE_B200_TC_WAIT_LIMIT lowers it (0 makes every wait
  // give up at once: the failure path is then exercised without a fault)
  ctx->tc_wait_limit = int64_t(1) << 26;
  if (const char *wl = getenv("ACE_B200_TC_WAIT_LIMIT")) {
    const long long v = atoll(wl);
    if (v >= 0 && v < ctx->tc_wait_limit) ctx->tc_wait_limit = v;
  }
  // tensor-core inference when the inputs fit one MMA K step (ACE_B200_MLP=fp32: CUDA cores)
  const char *menv = getenv("ACE_B200_MLP");
  ctx->mlp_tc = ctx->mlpD <= TC_K1 && ctx->mlpC <= TC_N3 && ctx->mlpC % 4 == 0 &&
                !(menv && std::string(menv) == "fp32");
  if (ctx->mlp_tc) {
    if (cudaFuncSetAttribute(mlp_fwd_tc_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin) !=
        cudaSuccess) {
      ctx->err = "cudaFuncSetAttribute failed";
      return ACE_ERR_CUDA;
    }
    int ot = 1;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ot, mlp_fwd_tc_kernel, 128, sizeof(TCSmem));
    // two CTAs per SM: their TC_COLS TMEM columns fill the SM's 512 and their
    // shared memory (sizeof(TCSmem) each) keeps a third out
    (void)ot;
    ctx->mlp_grid_tc = ctx->nsm * 2;
  }
  ctx->mlp_smem_f = fwd_smem(ctx);
  ctx->mlp_smem_b = bwd_smem(ctx);
  if (ctx->mlp_smem_f > (size_t)ctx->smem_optin || ctx->mlp_smem_b > (size_t)ctx->smem_optin) {
    ctx->err = "radial MLP too large for shared memory";
    return ACE_ERR_UNSUPPORTED;
  }
  if (cudaFuncSetAttribute(mlp_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin) !=
          cudaSuccess ||
      cudaFuncSetAttribute(mlp_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin) !=
          cudaSuccess) {
    ctx->err = "cudaFuncSetAttribute failed";
    return ACE_ERR_CUDA;
  }
  int of = 1, ob = 1;
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&of, mlp_fwd_kernel, NTF, ctx->mlp_smem_f);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&ob, mlp_bwd_kernel, NTB, ctx->mlp_smem_b);
  ctx->mlp_grid_f = ctx->nsm * std::max(of, 1);
  ctx->mlp_grid_b = ctx->nsm * std::max(ob, 1);
  return ACE_OK;
}

int mlp_forward(ace_ctx *ctx, int64_t nEnv, const int64_t *off, int64_t nNbr, const double *rr, const int32_t *sp,
                float *R, cudaStream_t st) {
  MLPArgs a = mlp_args(ctx);
  a.n = nNbr; a.off = off; a.nEnv = nEnv; a.rr = rr; a.sp = sp; a.R = R;
  const int64_t tiles = nNbr >= 0 ? (nNbr + NTF - 1) / NTF : ctx->mlp_grid_f;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, ctx->mlp_grid_f));
  void *args[] = {&a};
  cudaError_t e = cudaLaunchKernel((void *)mlp_fwd_kernel, dim3(grid), dim3(NTF), args, ctx->mlp_smem_f, st);
  ctx->launches += 1;
  if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return ACE_ERR_CUDA; }
  return ACE_OK;
}

// radial channels of every neighbour of the batch into the context's buffer
int learned_radials(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                    cudaStream_t st, bool infer) {
  int64_t nNbr = 0;
  if (cudaMemcpyAsync(&nNbr, off + nEnv, sizeof(int64_t), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    ctx->err = "reading the neighbour count failed";
    return ACE_ERR_CUDA;
  }
  if (nNbr < 0) { ctx->err = "negative neighbour count"; return ACE_ERR_INVALID; }
  if (nNbr > ctx->rext_cap) {
    if (ctx->d_Rext) cudaFree(ctx->d_Rext);
    ctx->d_Rext = nullptr;
    ctx->rext_cap = 0;
    const int64_t cap = std::max<int64_t>(nNbr, 1024);
    if (cudaMalloc(&ctx->d_Rext, (size_t)cap * 2 * ctx->mlpC * sizeof(float)) != cudaSuccess) {
      ctx->err = "radial buffer allocation failed";
      return ACE_ERR_ALLOC;
    }
    ctx->rext_cap = cap;
  }
  if (nNbr == 0) return ACE_OK;
  if (!ctx->mlp_tc || !infer) return mlp_forward(ctx, nEnv, off, nNbr, rr, sp, ctx->d_Rext, st);
  return mlp_infer(ctx, nEnv, off, nNbr, rr, sp, ctx->d_Rext, st);
}

// inference radials: tensor cores when the context allows them, else FP32
int mlp_infer(ace_ctx *ctx, int64_t nEnv, const int64_t *off, int64_t nNbr, const double *rr, const int32_t *sp,
              float *R, cudaStream_t st) {
  if (!ctx->mlp_tc) return mlp_forward(ctx, nEnv, off, nNbr, rr, sp, R, st);
  MLPArgs a = mlp_args(ctx);
  a.n = nNbr; a.off = off; a.nEnv = nEnv; a.rr = rr; a.sp = sp; a.R = R;
  const int64_t tiles = nNbr >= 0 ? (nNbr + 127) / 128 : ctx->mlp_grid_tc;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>(tiles, ctx->mlp_grid_tc));
  void *args[] = {&a};
  cudaError_t e = cudaLaunchKernel((void *)mlp_fwd_tc_kernel, dim3(grid), dim3(128), args, sizeof(TCSmem), st);
  ctx->launches += 1;
  if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return ACE_ERR_CUDA; }
  return ACE_OK;
}

}  // namespace ace

using namespace ace;

static int mfail(ace_ctx *ctx, int code, const char *why) {
  if (ctx) ctx->err = why;
  return code;
}

extern "C" int ace_set_radial_mlp(ace_ctx *ctx, const ace_radial_mlp *m) {
  if (!ctx || !m) return ACE_ERR_INVALID;
  if (m->version != 1) return mfail(ctx, ACE_ERR_INVALID, "unknown ace_radial_mlp version");
  if (ctx->nspecies != 1) return mfail(ctx, ACE_ERR_UNSUPPORTED, "the learned form needs a single-species spec");
  if (m->K != ctx->nR) return mfail(ctx, ACE_ERR_INVALID, "K must equal the spec's radial count");
  if (m->H != MLP_H) return mfail(ctx, ACE_ERR_UNSUPPORTED, "hidden width must be 64");
  if (m->Q < 1 || m->Q > MLP_MAXQ) return mfail(ctx, ACE_ERR_UNSUPPORTED, "Q out of range [1, 16]");
  if (m->nspecies < 1 || m->nspecies > MLP_MAXS) return mfail(ctx, ACE_ERR_UNSUPPORTED, "nspecies out of range [1, 8]");
  const int C = m->K * (ctx->L + 1);
  if (C > MLP_MAXC) return mfail(ctx, ACE_ERR_UNSUPPORTED, "K (L+1) above 512");
  if (!(m->tmax > ctx->tl)) return mfail(ctx, ACE_ERR_INVALID, "tmax must exceed the envelope root tl");
  const int D = m->Q + m->nspecies;
  const MLPOff o = mlp_off(MLP_H, D, C);
  if (!m->params || m->nparams != o.n) return mfail(ctx, ACE_ERR_INVALID, "nparams does not match the layout");
  for (int64_t i = 0; i < o.n; ++i)
    if (!std::isfinite(m->params[i])) return mfail(ctx, ACE_ERR_INVALID, "non-finite parameter");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return mfail(ctx, ACE_ERR_CUDA, "cudaSetDevice failed");
  const bool first = !ctx->learned;
  if (!first && (ctx->mlpC != C || ctx->mlpD != D)) return mfail(ctx, ACE_ERR_INVALID, "MLP shape changed");
  if (first) {
    // A entry (n, l, m) reads channel n + K l
    std::vector<int16_t> an(ctx->nA), aiy(ctx->nA);
    if (cudaMemcpy(an.data(), ctx->d_an, ctx->nA * sizeof(int16_t), cudaMemcpyDeviceToHost) != cudaSuccess ||
        cudaMemcpy(aiy.data(), ctx->d_aiy, ctx->nA * sizeof(int16_t), cudaMemcpyDeviceToHost) != cudaSuccess)
      return mfail(ctx, ACE_ERR_CUDA, "spec download failed");
    for (int i = 0; i < ctx->nA; ++i) {
      int l = (int)std::sqrt((double)aiy[i]);
      while (l * l > aiy[i]) --l;
      while ((l + 1) * (l + 1) <= aiy[i]) ++l;
      an[i] = (int16_t)(an[i] + m->K * l);
    }
    if (cudaMemcpy(ctx->d_an, an.data(), ctx->nA * sizeof(int16_t), cudaMemcpyHostToDevice) != cudaSuccess)
      return mfail(ctx, ACE_ERR_CUDA, "spec upload failed");
    if (cudaMalloc(&ctx->d_mlp, o.n * sizeof(float)) != cudaSuccess)
      return mfail(ctx, ACE_ERR_ALLOC, "parameter allocation failed");
  }
  if (cudaMemcpy(ctx->d_mlp, m->params, o.n * sizeof(float), cudaMemcpyHostToDevice) != cudaSuccess)
    return mfail(ctx, ACE_ERR_CUDA, "parameter upload failed");
  ctx->learned = true;
  ctx->mlpK = m->K; ctx->mlpQ = m->Q; ctx->mlpS = m->nspecies; ctx->mlpH = m->H; ctx->mlpC = C; ctx->mlpD = D;
  ctx->mlp_np = o.n;
  ctx->mlp_tmax = m->tmax;
  if (first) {
    int rc = kernels_prepare(ctx);
    if (rc) return rc;
    rc = mlp_prepare(ctx);
    if (rc) return rc;
  }
  return ACE_OK;
}

extern "C" int ace_radial_mlp_params(ace_ctx *ctx, float **d_params, int64_t *nparams) {
  if (!ctx || !d_params || !nparams) return ACE_ERR_INVALID;
  if (!ctx->learned) return mfail(ctx, ACE_ERR_INVALID, "no radial MLP set");
  *d_params = ctx->d_mlp;
  *nparams = ctx->mlp_np;
  return ACE_OK;
}

extern "C" int ace_radial_mlp_get_params(ace_ctx *ctx, float *params, int32_t flags) {
  if (!ctx || !params) return ACE_ERR_INVALID;
  if (!ctx->learned) return mfail(ctx, ACE_ERR_INVALID, "no radial MLP set");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return mfail(ctx, ACE_ERR_CUDA, "cudaSetDevice failed");
  const cudaMemcpyKind k = (flags & ACE_OUTPUTS_ON_DEVICE) ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
  if (cudaMemcpy(params, ctx->d_mlp, ctx->mlp_np * sizeof(float), k) != cudaSuccess)
    return mfail(ctx, ACE_ERR_CUDA, "parameter copy failed");
  return ACE_OK;
}

extern "C" int ace_radial_mlp_forward(ace_ctx *ctx, int64_t nNbr, const double *rr, const int32_t *species, float *R,
                                      void *stream) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!ctx->learned) return mfail(ctx, ACE_ERR_INVALID, "no radial MLP set");
  if (nNbr < 0 || (nNbr > 0 && (!rr || !R))) return mfail(ctx, ACE_ERR_INVALID, "NULL or negative argument");
  if (ctx->mlpS > 1 && nNbr > 0 && !species) return mfail(ctx, ACE_ERR_INVALID, "species required");
  if (nNbr == 0) return ACE_OK;
  return mlp_forward(ctx, 0, nullptr, nNbr, rr, ctx->mlpS > 1 ? species : nullptr, R, (cudaStream_t)stream);
}

extern "C" int ace_radial_mlp_infer(ace_ctx *ctx, int64_t nNbr, const double *rr, const int32_t *species, float *R,
                                    void *stream) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!ctx->learned) return mfail(ctx, ACE_ERR_INVALID, "no radial MLP set");
  if (nNbr < 0 || (nNbr > 0 && (!rr || !R))) return mfail(ctx, ACE_ERR_INVALID, "NULL or negative argument");
  if (ctx->mlpS > 1 && nNbr > 0 && !species) return mfail(ctx, ACE_ERR_INVALID, "species required");
  if (nNbr == 0) return ACE_OK;
  return mlp_infer(ctx, 0, nullptr, nNbr, rr, ctx->mlpS > 1 ? species : nullptr, R, (cudaStream_t)stream);
}

extern "C" int ace_radial_mlp_backward(ace_ctx *ctx, int64_t nNbr, const double *rr, const int32_t *species,
                                       const float *gR, const float *wj, float *gparams, void *stream) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!ctx->learned) return mfail(ctx, ACE_ERR_INVALID, "no radial MLP set");
  if (nNbr < 0 || !gparams || (nNbr > 0 && (!rr || !gR))) return mfail(ctx, ACE_ERR_INVALID, "NULL or negative argument");
  if (ctx->mlpS > 1 && nNbr > 0 && !species) return mfail(ctx, ACE_ERR_INVALID, "species required");
  if (nNbr == 0) return ACE_OK;
  MLPArgs a = mlp_args(ctx);
  a.n = nNbr; a.rr = rr; a.sp = ctx->mlpS > 1 ? species : nullptr; a.gR = gR; a.wj = wj; a.gW = gparams;
  const int grid = (int)std::max<int64_t>(1, std::min<int64_t>((nNbr + NTB - 1) / NTB, ctx->mlp_grid_b));
  void *args[] = {&a};
  cudaError_t e = cudaLaunchKernel((void *)mlp_bwd_kernel, dim3(grid), dim3(NTB), args, ctx->mlp_smem_b,
                                   (cudaStream_t)stream);
  ctx->launches += 1;
  if (e != cudaSuccess) return mfail(ctx, ACE_ERR_CUDA, cudaGetErrorString(e));
  return ACE_OK;
}

extern "C" int ace_energy_radial_adjoint(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                                         const int32_t *species, double *E, double *dEdrr, float *GR, void *stream) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!ctx->learned) return mfail(ctx, ACE_ERR_INVALID, "no radial MLP set");
  if (nEnv < 0 || (nEnv > 0 && (!offsets || !rr || !E || !GR)))
    return mfail(ctx, ACE_ERR_INVALID, "NULL or negative argument");
  if (ctx->mlpS > 1 && nEnv > 0 && !species) return mfail(ctx, ACE_ERR_INVALID, "species required");
  if (cudaSetDevice(ctx->device) != cudaSuccess) return mfail(ctx, ACE_ERR_CUDA, "cudaSetDevice failed");
  return launch_radial_adjoint(ctx, nEnv, offsets, rr, ctx->mlpS > 1 ? species : nullptr, E, dEdrr, GR,
                               (cudaStream_t)stream);
}

extern "C" int ace_adam_step(int64_t n, float *w, const float *g, float *m, float *v, float lr, float beta1,
                             float beta2, float eps, int32_t step, void *stream) {
  if (n < 0 || (n > 0 && (!w || !g || !m || !v)) || step < 1) return ACE_ERR_INVALID;
  if (n == 0) return ACE_OK;
  const float bc1 = 1.f - std::pow(beta1, (float)step), bc2 = 1.f - std::pow(beta2, (float)step);
  const int grid = (int)std::min<int64_t>((n + 255) / 256, 4096);
  adam_kernel<<<grid, 256, 0, (cudaStream_t)stream>>>(n, w, g, m, v, lr, beta1, beta2, eps, bc1, bc2);
  return cudaGetLastError() == cudaSuccess ? ACE_OK : ACE_ERR_CUDA;
}
