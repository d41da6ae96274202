// ace_kernels.cuh -- evaluation kernels of libace_b200.
//
// ef_kernel: one CTA per environment (grid-stride over environments).
//   phase 1  A_i = sum_j [mu_j == mu_i] R_{n_i}(r_j) Y_{l_i m_i}(rhat_j)
//            neighbours staged CH at a time: one thread per neighbour builds
//            R and Y in its shared-memory slab, then one thread per A entry
//            accumulates (src/product_1pbasis.jl:99-134).
//   phase 2  E = c~_0 + sum_k c~_k Re(prod_t A_{v_t}) and, for forces, the
//            adjoint dAco_v = sum_k c~_k dAA_k/dA_v by prefix/suffix
//            products (src/evaluator.jl:121-147,161-186; _AA_local_adjoints!,
//            src/pibasis.jl:338-390), accumulated with shared-memory atomics.
//   phase 3  g_j = sum_i Re(dAco_i (R'_{n_i} rhat_j Y_i + R_{n_i} grad Y_i))
//            with R', grad Y recomputed per neighbour instead of storing
//            dA (src/evaluator.jl:187-192).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_phi.cuh"

namespace ace {

struct EFArgs {
  int64_t nEnv;
  const int64_t *off;
  const double *rr;
  const int32_t *sp;
  double *E;
  double *G;
  const void *tab;
  int ntab, nR, L, pl, pr, tp;
  double tl, tr, r0;
  const int16_t *an, *aiy, *amu;
  int nA, nspecies;
  const uint8_t *ord;
  const uint16_t *idx;
  const void *ct;
  int64_t nAA;
  int has_const;
  int chunk;
  int *status;
  // basis path: write real(AA) for environments [e0, e0 + ldE) into AAout[k * ldE + e - e0]
  void *AAout;
  int64_t e0, ldE;
};

struct EFLayout {
  size_t tab, an, aiy, amu, A, D, pos, spc, slab, red, total;
  int slab_sz;
};

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

__host__ __device__ inline EFLayout ef_layout(int ntab, int nR, int L, int nA, int chunk, int tsize) {
  EFLayout l;
  size_t o = 0;
  l.tab = o; o = al16(o + (size_t)ntab * tsize);
  l.an = o; o = al16(o + (size_t)nA * 2);
  l.aiy = o; o = al16(o + (size_t)nA * 2);
  l.amu = o; o = al16(o + (size_t)nA * 2);
  l.A = o; o = al16(o + (size_t)nA * 2 * tsize);
  l.D = o; o = al16(o + (size_t)nA * 2 * tsize);
  l.pos = o; o = al16(o + (size_t)chunk * 4 * tsize);
  l.spc = o; o = al16(o + (size_t)chunk * 4);
  l.slab_sz = 2 * nR + 2 * size_p(L) + 8 * size_y(L);
  l.slab = o; o = al16(o + (size_t)chunk * l.slab_sz * tsize);
  l.red = o; o = al16(o + 32 * 8);
  l.total = o;
  return l;
}

template <typename T> __device__ __forceinline__ void atomic_add_c(cpx<T> *p, cpx<T> v) {
  atomicAdd(&p->re, v.re);
  atomicAdd(&p->im, v.im);
}

// One AA function: returns c * Re(prod), and with GRAD adds c * dAA/dA_{v_t}
// into D[v_t] (prefix products pre[t] times suffix products).
template <typename T, int MAXORD, bool GRAD>
__device__ __forceinline__ T aa_term(int ord, const int (&v)[MAXORD], const cpx<T> *A, T c, cpx<T> *D) {
  cpx<T> a[MAXORD], pre[MAXORD];
  cpx<T> fwd = {T(1), T(0)};
#pragma unroll
  for (int t = 0; t < MAXORD; ++t) {
    pre[t] = fwd;
    if (t < ord) {
      a[t] = A[v[t]];
      fwd = (t == 0) ? a[t] : cmul(fwd, a[t]);
    }
  }
  if (GRAD) {
    cpx<T> bwd = {T(1), T(0)};
#pragma unroll
    for (int t = MAXORD - 1; t >= 0; --t) {
      if (t < ord) {
        const cpx<T> d = (t == ord - 1) ? pre[t] : cmul(pre[t], bwd);
        atomic_add_c(&D[v[t]], cscale(d, c));
        bwd = (t == ord - 1) ? a[t] : cmul(bwd, a[t]);
      }
    }
  }
  return c * fwd.re;
}

template <typename T>
__device__ __forceinline__ double block_sum(double v, double *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  if (lane == 0) red[w] = v;
  __syncthreads();
  double s = 0.0;
  if (w == 0) {
    s = lane < nw ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  }
  __syncthreads();
  return s;  // valid in thread 0
}

// modes: 0 = energy, 1 = energy + forces, 2 = real(AA) to AAout (basis path)
template <typename T, int MAXORD, int MODE>
__global__ void __launch_bounds__(256) ef_kernel(EFArgs a) {
  constexpr bool GRAD = (MODE == 1);
  extern __shared__ __align__(16) unsigned char sm[];
  const EFLayout lay = ef_layout(a.ntab, a.nR, a.L, a.nA, a.chunk, sizeof(T));
  T *tab = (T *)(sm + lay.tab);
  int16_t *s_an = (int16_t *)(sm + lay.an);
  int16_t *s_aiy = (int16_t *)(sm + lay.aiy);
  int16_t *s_amu = (int16_t *)(sm + lay.amu);
  cpx<T> *sA = (cpx<T> *)(sm + lay.A);
  cpx<T> *sD = (cpx<T> *)(sm + lay.D);
  T *spos = (T *)(sm + lay.pos);
  int *ssp = (int *)(sm + lay.spc);
  T *slab = (T *)(sm + lay.slab);
  double *red = (double *)(sm + lay.red);
  const int tid = threadIdx.x, bs = blockDim.x;
  const int SS = lay.slab_sz;
  const int szP = size_p(a.L);

  for (int i = tid; i < a.ntab; i += bs) tab[i] = ((const T *)a.tab)[i];
  for (int i = tid; i < a.nA; i += bs) { s_an[i] = a.an[i]; s_aiy[i] = a.aiy[i]; s_amu[i] = a.amu[i]; }
  __syncthreads();
  Tables<T> tb;
  tb.rA = tab; tb.rB = tab + a.nR; tb.rC = tab + 2 * a.nR;
  tb.alpA = tab + 3 * a.nR; tb.alpB = tab + 3 * a.nR + szP;
  tb.nR = a.nR; tb.L = a.L; tb.pl = a.pl; tb.pr = a.pr; tb.tp = a.tp;
  tb.tl = T(a.tl); tb.tr = T(a.tr); tb.r0 = T(a.r0);
  const T *ct = (const T *)a.ct;
  const int64_t ntot = a.off[a.nEnv];

  for (int64_t e = blockIdx.x; e < a.nEnv; e += gridDim.x) {
    const int64_t o0 = a.off[e], o1 = a.off[e + 1];
    if (o0 < 0 || o1 < o0 || o1 > ntot) {
      if (tid == 0) {
        atomicOr(a.status, ACE_STATUS_BAD_OFFSETS);
        if (MODE != 2) a.E[e] = __longlong_as_double(0x7ff8000000000000ll);
      }
      continue;
    }
    const int J = (int)(o1 - o0);
    for (int i = tid; i < a.nA; i += bs) sA[i] = {T(0), T(0)};
    // ---------------- phase 1: A
    for (int c0 = 0; c0 < J; c0 += a.chunk) {
      const int nc = min(a.chunk, J - c0);
      __syncthreads();
      if (tid < nc) {
        const int64_t j = o0 + c0 + tid;
        const T x = T(a.rr[3 * j]), y = T(a.rr[3 * j + 1]), z = T(a.rr[3 * j + 2]);
        int s = 0;
        if (a.nspecies > 1) {
          s = a.sp[j];
          if (s < 0 || s >= a.nspecies) { atomicOr(a.status, ACE_STATUS_BAD_SPECIES); s = -1; }
        }
        ssp[tid] = s;
        const T r = sqrt(x * x + y * y + z * z);
        if (!(r > T(0)) || !isfinite(r)) atomicOr(a.status, ACE_STATUS_BAD_POSITION);
        T *sl = slab + (size_t)tid * SS;
        radial_eval<T, false>(tb, r, sl, nullptr);
        sh_eval<T, false>(tb, x, y, z, sl + 2 * a.nR, sl + 2 * a.nR + szP,
                          (cpx<T> *)(sl + 2 * a.nR + 2 * szP), nullptr);
      }
      __syncthreads();
      for (int i = tid; i < a.nA; i += bs) {
        const int n = s_an[i], iy = s_aiy[i], mu = s_amu[i];
        cpx<T> acc = sA[i];
        for (int jj = 0; jj < nc; ++jj) {
          if (a.nspecies > 1 && ssp[jj] != mu) continue;
          const T *sl = slab + (size_t)jj * SS;
          const cpx<T> Y = ((const cpx<T> *)(sl + 2 * a.nR + 2 * szP))[iy];
          acc = cadd(acc, cscale(Y, sl[n]));
        }
        sA[i] = acc;
      }
    }
    if (GRAD)
      for (int i = tid; i < a.nA; i += bs) sD[i] = {T(0), T(0)};
    __syncthreads();
    // ---------------- phase 2: AA products (+ adjoint)
    if (MODE == 2) {
      T *AAout = (T *)a.AAout;
      const int64_t col = e - a.e0;
      for (int64_t k = tid; k < a.nAA; k += bs) {
        const int ord = a.ord[k];
        cpx<T> p = {T(1), T(0)};
        for (int t = 0; t < ord; ++t) p = cmul(p, sA[a.idx[(size_t)t * a.nAA + k]]);
        AAout[k * a.ldE + col] = p.re;
      }
      __syncthreads();
      continue;
    }
    T eloc = T(0);
    for (int64_t k = tid + a.has_const; k < a.nAA; k += bs) {
      const int ord = a.ord[k];
      int v[MAXORD];
#pragma unroll
      for (int t = 0; t < MAXORD; ++t) v[t] = (t < ord) ? (int)a.idx[(size_t)t * a.nAA + k] : 0;
      eloc += aa_term<T, MAXORD, GRAD>(ord, v, sA, ct[k], sD);
    }
    const double esum = block_sum<T>((double)eloc, red);
    if (tid == 0) a.E[e] = (a.has_const ? (double)ct[0] : 0.0) + esum;
    if (!GRAD) continue;
    // ---------------- phase 3: forces
    const int lane = tid & 31, w = tid >> 5, nw = bs >> 5;
    for (int c0 = 0; c0 < J; c0 += a.chunk) {
      const int nc = min(a.chunk, J - c0);
      __syncthreads();
      if (tid < nc) {
        const int64_t j = o0 + c0 + tid;
        const T x = T(a.rr[3 * j]), y = T(a.rr[3 * j + 1]), z = T(a.rr[3 * j + 2]);
        int s = 0;
        if (a.nspecies > 1) {
          s = a.sp[j];
          if (s < 0 || s >= a.nspecies) s = -1;
        }
        ssp[tid] = s;
        const T r = sqrt(x * x + y * y + z * z);
        spos[4 * tid + 0] = x / r; spos[4 * tid + 1] = y / r; spos[4 * tid + 2] = z / r;
        T *sl = slab + (size_t)tid * SS;
        radial_eval<T, true>(tb, r, sl, sl + a.nR);
        sh_eval<T, true>(tb, x, y, z, sl + 2 * a.nR, sl + 2 * a.nR + szP,
                         (cpx<T> *)(sl + 2 * a.nR + 2 * szP),
                         (cpx<T> *)(sl + 2 * a.nR + 2 * szP) + size_y(a.L));
      }
      __syncthreads();
      for (int jj = w; jj < nc; jj += nw) {
        const T *sl = slab + (size_t)jj * SS;
        const cpx<T> *Y = (const cpx<T> *)(sl + 2 * a.nR + 2 * szP);
        const cpx<T> *dY = Y + size_y(a.L);
        const int s = ssp[jj];
        T g0 = T(0), g1 = T(0), g2 = T(0), gr = T(0);
        for (int i = lane; i < a.nA; i += 32) {
          if (a.nspecies > 1 && s_amu[i] != s) continue;
          const int n = s_an[i], iy = s_aiy[i];
          const cpx<T> d = sD[i];
          const T R = sl[n], dR = sl[a.nR + n];
          const cpx<T> y0 = Y[iy];
          gr += dR * (d.re * y0.re - d.im * y0.im);
          const cpx<T> *dy = dY + 3 * iy;
          g0 += R * (d.re * dy[0].re - d.im * dy[0].im);
          g1 += R * (d.re * dy[1].re - d.im * dy[1].im);
          g2 += R * (d.re * dy[2].re - d.im * dy[2].im);
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          g0 += __shfl_xor_sync(0xffffffffu, g0, o);
          g1 += __shfl_xor_sync(0xffffffffu, g1, o);
          g2 += __shfl_xor_sync(0xffffffffu, g2, o);
          gr += __shfl_xor_sync(0xffffffffu, gr, o);
        }
        if (lane == 0) {
          const int64_t j = o0 + c0 + jj;
          a.G[3 * j + 0] = (double)(gr * spos[4 * jj + 0] + g0);
          a.G[3 * j + 1] = (double)(gr * spos[4 * jj + 1] + g1);
          a.G[3 * j + 2] = (double)(gr * spos[4 * jj + 2] + g2);
        }
      }
    }
    __syncthreads();
  }
}

// B[e * nB + b] = sum_k U[b, k] AA[k * ldE + e - e0]  (genmul!, src/symmbasis.jl:248-264)
template <typename T>
__global__ void ub_kernel(int64_t ne, int64_t e0, int64_t ldE, int64_t nB, const int64_t *Uptr,
                          const int32_t *Uidx, const T *Uval, const T *AA, double *B) {
  const int64_t e = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (e >= ne) return;
  for (int64_t b = blockIdx.y; b < nB; b += gridDim.y) {
    T acc = T(0);
    for (int64_t k = Uptr[b]; k < Uptr[b + 1]; ++k) acc += Uval[k] * AA[(int64_t)Uidx[k] * ldE + e];
    B[(e0 + e) * nB + b] = (double)acc;
  }
}

// ------------------------------------------------------------------ host side

template <typename T, int MODE>
static void *pick_ef(int maxord) {
  if (maxord <= 2) return (void *)ef_kernel<T, 2, MODE>;
  if (maxord <= 4) return (void *)ef_kernel<T, 4, MODE>;
  if (maxord <= 6) return (void *)ef_kernel<T, 6, MODE>;
  return (void *)ef_kernel<T, 8, MODE>;
}

static void *ef_func(const ace_ctx *ctx, int mode) {
  const bool dbl = (ctx->prec == ACE_PREC_FP64);
  switch (mode) {
    case 0: return dbl ? pick_ef<double, 0>(ctx->maxord) : pick_ef<float, 0>(ctx->maxord);
    case 1: return dbl ? pick_ef<double, 1>(ctx->maxord) : pick_ef<float, 1>(ctx->maxord);
    default: return dbl ? pick_ef<double, 2>(ctx->maxord) : pick_ef<float, 2>(ctx->maxord);
  }
}

inline int kernels_prepare(ace_ctx *ctx) {
  const int tsize = (ctx->prec == ACE_PREC_FP64) ? 8 : 4;
  // neighbour chunk: as many as fit in ~96 KB of slabs (at most 64, at least 1)
  const int slab = (2 * ctx->nR + 2 * size_p(ctx->L) + 8 * size_y(ctx->L)) * tsize;
  int chunk = (int)std::min<long>(64, std::max<long>(1, (96 * 1024) / slab));
  EFLayout lay = ef_layout(ctx->ntab, ctx->nR, ctx->L, ctx->nA, chunk, tsize);
  while (lay.total > (size_t)ctx->smem_optin && chunk > 1) {
    chunk /= 2;
    lay = ef_layout(ctx->ntab, ctx->nR, ctx->L, ctx->nA, chunk, tsize);
  }
  if (lay.total > (size_t)ctx->smem_optin) {
    ctx->err = "spec too large for shared memory";
    return ACE_ERR_UNSUPPORTED;
  }
  ctx->ef_chunk = chunk;
  ctx->ef_smem = lay.total;
  ctx->ef_block = 256;
  int occ = 1;
  for (int mode = 0; mode < 3; ++mode) {
    void *f = ef_func(ctx, mode);
    if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)lay.total) != cudaSuccess) {
      ctx->err = "cudaFuncSetAttribute failed";
      return ACE_ERR_CUDA;
    }
    if (mode == 1) cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, f, ctx->ef_block, lay.total);
  }
  ctx->ef_grid = ctx->nsm * std::max(occ, 1);
  return ACE_OK;
}

inline EFArgs make_args(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                        double *E, double *G) {
  EFArgs a;
  const bool dbl = (ctx->prec == ACE_PREC_FP64);
  a.nEnv = nEnv; a.off = off; a.rr = rr; a.sp = sp; a.E = E; a.G = G;
  a.tab = dbl ? (const void *)ctx->d_tabD : (const void *)ctx->d_tabF;
  a.ntab = ctx->ntab; a.nR = ctx->nR; a.L = ctx->L; a.pl = ctx->pl; a.pr = ctx->pr; a.tp = ctx->tp;
  a.tl = ctx->tl; a.tr = ctx->tr; a.r0 = ctx->r0;
  a.an = ctx->d_an; a.aiy = ctx->d_aiy; a.amu = ctx->d_amu;
  a.nA = ctx->nA; a.nspecies = ctx->nspecies;
  a.ord = ctx->d_ord; a.idx = ctx->d_idx;
  a.ct = dbl ? (const void *)ctx->d_ctD : (const void *)ctx->d_ctF;
  a.nAA = ctx->nAA; a.has_const = ctx->has_const ? 1 : 0;
  a.chunk = ctx->ef_chunk; a.status = ctx->d_status;
  a.AAout = nullptr; a.e0 = 0; a.ldE = 0;
  return a;
}

inline int launch_energy_forces(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr,
                                const int32_t *sp, double *E, double *G, cudaStream_t st) {
  if (nEnv == 0) return ACE_OK;
  EFArgs a = make_args(ctx, nEnv, off, rr, sp, E, G);
  void *f = ef_func(ctx, G ? 1 : 0);
  const int grid = (int)std::min<int64_t>(nEnv, ctx->ef_grid);
  void *args[] = {&a};
  cudaError_t e = cudaLaunchKernel(f, dim3(grid), dim3(ctx->ef_block), args, ctx->ef_smem, st);
  ctx->launches += 1;
  if (e != cudaSuccess) { ctx->err = cudaGetErrorString(e); return ACE_ERR_CUDA; }
  return ACE_OK;
}

inline int ensure_scratch(ace_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->scratch_bytes) return ACE_OK;
  if (ctx->d_scratch) { cudaFree(ctx->d_scratch); ctx->d_scratch = nullptr; ctx->scratch_bytes = 0; }
  if (cudaMalloc(&ctx->d_scratch, bytes) != cudaSuccess) { ctx->err = "scratch allocation failed"; return ACE_ERR_ALLOC; }
  ctx->scratch_bytes = bytes;
  return ACE_OK;
}

inline int launch_basis(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                        double *B, double *dB, cudaStream_t st) {
  if (dB) { ctx->err = "dB is produced by the dB path"; return ACE_ERR_UNSUPPORTED; }
  if (nEnv == 0) return ACE_OK;
  const bool dbl = (ctx->prec == ACE_PREC_FP64);
  const size_t ts = dbl ? 8 : 4;
  // environments per pass so that the AA scratch stays within 512 MB
  int64_t per = std::max<int64_t>(1, (int64_t)((512ull << 20) / (ctx->nAA * ts)));
  per = std::min<int64_t>(per, nEnv);
  int rc = ensure_scratch(ctx, (size_t)per * ctx->nAA * ts);
  if (rc) return rc;
  void *f = ef_func(ctx, 2);
  for (int64_t e0 = 0; e0 < nEnv; e0 += per) {
    const int64_t ne = std::min(per, nEnv - e0);
    EFArgs a = make_args(ctx, e0 + ne, off, rr, sp, nullptr, nullptr);
    a.AAout = ctx->d_scratch; a.e0 = e0; a.ldE = ne;
    // restrict the grid-stride loop to [e0, e0 + ne): shift via the first block index
    // (blocks start at e0 by offsetting the environment pointer view)
    const int grid = (int)std::min<int64_t>(ne, ctx->ef_grid);
    EFArgs a2 = a;
    a2.nEnv = ne;
    a2.off = off + e0;   // environment e (local) reads off[e0 + e]
    a2.e0 = 0;
    void *args[] = {&a2};
    // off + e0 shifts the CSR view; ntot check uses off[nEnv] of the view, which is the true end
    cudaError_t err = cudaLaunchKernel(f, dim3(grid), dim3(ctx->ef_block), args, ctx->ef_smem, st);
    ctx->launches += 1;
    if (err != cudaSuccess) { ctx->err = cudaGetErrorString(err); return ACE_ERR_CUDA; }
    dim3 g2((unsigned)((ne + 127) / 128), (unsigned)std::min<int64_t>(ctx->nB, 65535));
    if (dbl)
      ub_kernel<double><<<g2, 128, 0, st>>>(ne, e0, ne, ctx->nB, ctx->d_Uptr, ctx->d_Uidx, ctx->d_UvalD,
                                             (const double *)ctx->d_scratch, B);
    else
      ub_kernel<float><<<g2, 128, 0, st>>>(ne, e0, ne, ctx->nB, ctx->d_Uptr, ctx->d_Uidx, ctx->d_UvalF,
                                            (const float *)ctx->d_scratch, B);
    ctx->launches += 1;
    err = cudaGetLastError();
    if (err != cudaSuccess) { ctx->err = cudaGetErrorString(err); return ACE_ERR_CUDA; }
  }
  return ACE_OK;
}

}  // namespace ace
