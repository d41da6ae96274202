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
#include <vector>

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

static MLPArgs mlp_args(const ace_ctx *ctx) {
  MLPArgs a{};
  a.W = ctx->d_mlp;
  a.D = ctx->mlpD; a.Q = ctx->mlpQ; a.S = ctx->mlpS; a.C = ctx->mlpC;
  a.a0 = (float)(1.0 + ctx->r0);
  a.tl = (float)ctx->tl; a.tr = (float)ctx->tr;
  a.xs = (float)(2.0 / (ctx->mlp_tmax - ctx->tl));
  a.tp = ctx->tp; a.pl = ctx->pl; a.pr = ctx->pr;
  a.status = ctx->d_status;
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
  ctx->mlp_smem_f = fwd_smem(ctx);
  ctx->mlp_smem_b = bwd_smem(ctx);
  if (ctx->mlp_smem_f > (size_t)ctx->smem_optin || ctx->mlp_smem_b > (size_t)ctx->smem_optin) {
    ctx->err = "radial MLP too large for shared memory";
    return ACE_ERR_UNSUPPORTED;
  }
  if (cudaFuncSetAttribute(mlp_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->mlp_smem_f) !=
          cudaSuccess ||
      cudaFuncSetAttribute(mlp_bwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)ctx->mlp_smem_b) !=
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
                    cudaStream_t st) {
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
  return mlp_forward(ctx, nEnv, off, nNbr, rr, sp, ctx->d_Rext, st);
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
