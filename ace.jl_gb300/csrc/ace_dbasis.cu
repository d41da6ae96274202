// ace_dbasis.cu -- derivatives of the symmetric basis on the GPU:
//
//   dB[j, b, a] = dB_b / d rr_j[a]     (SymmetricBasis evaluate_ed / evaluate_d,
//                                        src/symmbasis.jl:322-334; grad_params_config,
//                                        src/linearmodel.jl:127-128)
//   out[e, b]   = sum_{j in e, a} w[j, a] dB_b / d rr_j[a]
//                                       (adjoint_EVAL_D, src/evaluator.jl:204-244)
//
// Per environment (one CTA): A (phase 1 of the energy kernel), then per
// neighbour chunk the 1p-basis gradients dphi_v(r_j) = R'_n rhat Y_lm + R_n grad Y_lm
// (cYlm_ed!, src/polynomials/sphericalharmonics.jl:410-443) in a shared slab;
// one thread per AA function k forms the local adjoints dAA_k/dA_{v_t}
// (_AA_local_adjoints!, src/pibasis.jl:338-390) and contracts them:
//   dAA[k, j, a] = Re(sum_t adj_t dphi_{v_t}(r_j)[a])          (_evaluate_ed!, :402-432)
//   dAAw[k]      = Re(sum_t adj_t dAw_{v_t}),  dAw_v = sum_j w_j . dphi_v(r_j)
// into a scratch matrix; B-rows follow from U (genmul!, src/symmbasis.jl:248-264).
#include <cuda_runtime.h>

#include <algorithm>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_kernels.cuh"

namespace ace {

struct DArgs {
  EFArgs a;
  const double *w;     // adjoint weights (3 per neighbour) or NULL for dB
  int64_t jbase;       // global index of the pass's first neighbour
  int64_t ld;          // scratch leading dimension (columns)
  int chunk;           // neighbours per slab pass
};

template <typename T, bool DB>
__global__ void __launch_bounds__(256) daa_kernel(DArgs d) {
  const EFArgs &a = d.a;
  extern __shared__ __align__(16) unsigned char sm[];
  const EFLayout lay = ef_layout(a.ntab, a.nRs, a.L, a.nA, d.chunk, d.chunk, 0, 256, sizeof(T), sizeof(T), true);
  T *tab = (T *)(sm + lay.tabE);
  int16_t *s_an = (int16_t *)(sm + lay.an);
  int16_t *s_aiy = (int16_t *)(sm + lay.aiy);
  int16_t *s_amu = (int16_t *)(sm + lay.amu);
  cpx<T> *AE = (cpx<T> *)(sm + lay.AE);
  cpx<T> *Dw = (cpx<T> *)(sm + lay.D);
  T *spos = (T *)(sm + lay.pos);
  int *ssp = (int *)(sm + lay.spc);
  T *slab = (T *)(sm + lay.slab);
  const int tid = threadIdx.x, nt = blockDim.x;
  const int nY = size_y(a.L);
  const int SG = lay.slabG;
  for (int i = tid; i < a.ntab; i += nt) tab[i] = load_table<T>(a.tabE, i);
  for (int i = tid; i < a.nA; i += nt) { s_an[i] = a.an[i]; s_aiy[i] = a.aiy[i]; s_amu[i] = a.amu[i]; }
  __syncthreads();
  Tables<T> tb;
  tb.bind(tab, a.nR, a.L, a.pl, a.pr, a.tp);
  const int64_t ntot = a.off[a.nEnv];
  T *out = (T *)a.AAout;
  const int K = 8;  // local adjoint storage (maxord <= 6)
  for (int64_t e = blockIdx.x; e < a.nEnv; e += gridDim.x) {
    const int64_t o0 = a.off[e], o1 = a.off[e + 1];
    if (o0 < 0 || o1 < o0 || o1 > ntot) {
      if (tid == 0) atomicOr(a.status, ACE_STATUS_BAD_OFFSETS);
      continue;
    }
    const int J = (int)(o1 - o0);
    build_A<T>(a, tb, o0, J, d.chunk, lay.slabE, s_an, s_aiy, s_amu, ssp, slab, AE);
    if (!DB)
      for (int i = tid; i < a.nA; i += nt) Dw[i] = {T(0), T(0)};
    const int LP1 = a.L + 1;
    const int cj = tid / LP1, cm = tid - cj * LP1;
    for (int c0 = 0; c0 < J; c0 += d.chunk) {
      const int nc = min(d.chunk, J - c0);
      __syncthreads();
      if (cj < nc) {
        const int64_t j = o0 + c0 + cj;
        const T x = T(a.rr[3 * j]), y = T(a.rr[3 * j + 1]), z = T(a.rr[3 * j + 2]);
        const Angles<T> g = angles(x, y, z);
        T *sl = slab + (size_t)cj * SG;
        cpx<T> *Y = (cpx<T> *)(sl + 2 * a.nRs);
        cpx<T> *dY = Y + nY;
        if (a.Rext) {
          const float *rx = a.Rext + (size_t)j * 2 * a.nRs;
          for (int n = cm; n < a.nRs; n += LP1) {
            sl[n] = T(rx[n]);
            sl[a.nRs + n] = T(rx[a.nRs + n]);
          }
        }
        if (cm == 0) {
          int s = 0;
          if (a.nspecies > 1) {
            s = a.sp[j];
            if (s < 0 || s >= a.nspecies) s = -1;
          }
          ssp[cj] = s;
          const T ux = x / g.r, uy = y / g.r, uz = z / g.r;
          spos[4 * cj + 0] = ux; spos[4 * cj + 1] = uy; spos[4 * cj + 2] = uz;
          if (!DB) spos[4 * cj + 3] = T(d.w[3 * j]) * ux + T(d.w[3 * j + 1]) * uy + T(d.w[3 * j + 2]) * uz;
          if (!a.Rext) radial_eval<T, true>(tb, g.r, sl, sl + a.nRs);
        }
        sh_col_grad<T>(tb, g, cm, Y, dY);
        if (!DB) {
          // contract the weights into this column's entries: dY[.][0] <- w . grad Y
          const T w0 = T(d.w[3 * j]), w1 = T(d.w[3 * j + 1]), w2 = T(d.w[3 * j + 2]);
          for (int l = cm; l <= a.L; ++l)
            for (int sg = (cm == 0 ? 1 : -1); sg <= 1; sg += 2) {
              cpx<T> *q = dY + 3 * idx_y(l, sg * cm);
              q[0] = {w0 * q[0].re + w1 * q[1].re + w2 * q[2].re, w0 * q[0].im + w1 * q[1].im + w2 * q[2].im};
            }
        }
      }
      __syncthreads();
      if (!DB) {
        for (int i = tid; i < a.nA; i += nt) {
          const int n = s_an[i], iy = s_aiy[i], mu = s_amu[i];
          cpx<T> acc = Dw[i];
          for (int jj = 0; jj < nc; ++jj) {
            if (a.nspecies > 1 && ssp[jj] != mu) continue;
            const T *sl = slab + (size_t)jj * SG;
            const cpx<T> *Y = (const cpx<T> *)(sl + 2 * a.nRs);
            const cpx<T> g = (Y + nY)[3 * iy];
            const T dRs = sl[a.nRs + n] * spos[4 * jj + 3];
            acc = cadd(acc, cadd(cscale(Y[iy], dRs), cscale(g, sl[n])));
          }
          Dw[i] = acc;
        }
      } else {
        for (int64_t k = tid; k < a.nAA; k += nt) {
          const int ord = a.ord[k];
          int v[K];
          cpx<T> adj[K];
          for (int t = 0; t < ord; ++t) v[t] = a.idx[(size_t)t * a.nAA + k];
          // adj_t = prod_{s != t} A_{v_s} (prefix/suffix)
          cpx<T> pre = {T(1), T(0)};
          for (int t = 0; t < ord; ++t) { adj[t] = pre; pre = cmul(pre, AE[v[t]]); }
          cpx<T> suf = {T(1), T(0)};
          for (int t = ord - 1; t >= 0; --t) { adj[t] = cmul(adj[t], suf); suf = cmul(suf, AE[v[t]]); }
          for (int jj = 0; jj < nc; ++jj) {
            const T *sl = slab + (size_t)jj * SG;
            const cpx<T> *Y = (const cpx<T> *)(sl + 2 * a.nRs);
            const cpx<T> *dY = Y + nY;
            const int sp = ssp[jj];
            T g0 = T(0), g1 = T(0), g2 = T(0);
            for (int t = 0; t < ord; ++t) {
              const int vv = v[t];
              if (a.nspecies > 1 && s_amu[vv] != sp) continue;
              const int n = s_an[vv], iy = s_aiy[vv];
              const cpx<T> q = adj[t];
              const T R = sl[n], dR = sl[a.nRs + n];
              const T ry = q.re * Y[iy].re - q.im * Y[iy].im;
              const cpx<T> *g = dY + 3 * iy;
              g0 += dR * spos[4 * jj + 0] * ry + R * (q.re * g[0].re - q.im * g[0].im);
              g1 += dR * spos[4 * jj + 1] * ry + R * (q.re * g[1].re - q.im * g[1].im);
              g2 += dR * spos[4 * jj + 2] * ry + R * (q.re * g[2].re - q.im * g[2].im);
            }
            const int64_t col = 3 * (o0 + c0 + jj - d.jbase);
            out[k * d.ld + col + 0] = g0;
            out[k * d.ld + col + 1] = g1;
            out[k * d.ld + col + 2] = g2;
          }
        }
      }
    }
    __syncthreads();
    if (!DB) {
      for (int64_t k = tid; k < a.nAA; k += nt) {
        const int ord = a.ord[k];
        T acc = T(0);
        if (ord > 0) {
          int v[K];
          cpx<T> adj[K];
          for (int t = 0; t < ord; ++t) v[t] = a.idx[(size_t)t * a.nAA + k];
          cpx<T> pre = {T(1), T(0)};
          for (int t = 0; t < ord; ++t) { adj[t] = pre; pre = cmul(pre, AE[v[t]]); }
          cpx<T> suf = {T(1), T(0)};
          for (int t = ord - 1; t >= 0; --t) { adj[t] = cmul(adj[t], suf); suf = cmul(suf, AE[v[t]]); }
          for (int t = 0; t < ord; ++t) acc += Dw[v[t]].re * adj[t].re - Dw[v[t]].im * adj[t].im;
        }
        out[k * d.ld + e] = acc;
      }
      __syncthreads();
    }
  }
}

// out[col -> (row, axis)]: dB[((jbase + col/3) * nB + b) * 3 + col % 3] = sum_k U[b,k] S[k*ld + col]
template <typename T>
__global__ void udb_kernel(int64_t ncol, int64_t jbase, int64_t ld, int64_t nB, const int64_t *Uptr,
                           const int32_t *Uidx, const T *Uval, const T *S, double *dB) {
  const int64_t col = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (col >= ncol) return;
  const int64_t j = jbase + col / 3, ax = col % 3;
  for (int64_t b = blockIdx.y; b < nB; b += gridDim.y) {
    T acc = T(0);
    for (int64_t k = Uptr[b]; k < Uptr[b + 1]; ++k) acc += Uval[k] * S[(int64_t)Uidx[k] * ld + col];
    dB[(j * nB + b) * 3 + ax] = (double)acc;
  }
}

static int ensure_scratch_d(ace_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->scratch_bytes) return ACE_OK;
  if (ctx->d_scratch) { cudaFree(ctx->d_scratch); ctx->d_scratch = nullptr; ctx->scratch_bytes = 0; }
  if (cudaMalloc(&ctx->d_scratch, bytes) != cudaSuccess) { ctx->err = "scratch allocation failed"; return ACE_ERR_ALLOC; }
  ctx->scratch_bytes = bytes;
  return ACE_OK;
}

template <typename T, bool DB>
static int run_daa(ace_ctx *ctx, int64_t nEnv, const int64_t *off_d, const int64_t *off_h, const double *rr,
                   const int32_t *sp, const double *w, double *out, cudaStream_t st) {
  const size_t ts = sizeof(T);
  const int nRs = ctx->learned ? ctx->mlpC : ctx->nR;
  const int slabG = (2 * nRs + 8 * size_y(ctx->L)) * (int)ts;
  int chunk = std::max(1, std::min(std::min(32, 256 / (ctx->L + 1)), (48 * 1024) / slabG));
  EFLayout lay = ef_layout(ctx->ntab, nRs, ctx->L, ctx->nA, chunk, chunk, 0, 256, (int)ts, (int)ts, true);
  if (ctx->learned) {
    int rc = learned_radials(ctx, nEnv, off_d, rr, sp, st);
    if (rc) return rc;
  }
  void *f = (void *)daa_kernel<T, DB>;
  if (cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, ctx->smem_optin) != cudaSuccess) {
    ctx->err = "cudaFuncSetAttribute failed";
    return ACE_ERR_CUDA;
  }
  const size_t budget = 512ull << 20;
  int64_t e0 = 0;
  while (e0 < nEnv) {
    // environments per pass: scratch columns (envs, or 3 x neighbours) within the budget
    int64_t e1 = e0, cols = 0;
    while (e1 < nEnv) {
      const int64_t add = DB ? 3 * (off_h[e1 + 1] - off_h[e1]) : 1;
      if (e1 > e0 && (size_t)(cols + add) * ctx->nAA * ts > budget) break;
      cols += add;
      ++e1;
    }
    const int64_t ne = e1 - e0;
    if (cols == 0) { e0 = e1; continue; }
    int rc = ensure_scratch_d(ctx, (size_t)cols * ctx->nAA * ts);
    if (rc) return rc;
    DArgs d;
    d.a = make_args(ctx, ne, off_d + e0, rr, sp, nullptr, nullptr);
    d.a.AAout = ctx->d_scratch;
    d.a.tabE = (sizeof(T) == 8) ? (const void *)ctx->d_tabD : (const void *)ctx->d_tabF;
    d.w = w;
    d.jbase = DB ? off_h[e0] : 0;
    d.ld = cols;
    d.chunk = chunk;
    const int grid = (int)std::min<int64_t>(ne, 4 * ctx->nsm);
    void *args[] = {&d};
    cudaError_t err = cudaLaunchKernel(f, dim3(grid), dim3(256), args, lay.total, st);
    ctx->launches += 1;
    if (err != cudaSuccess) { ctx->err = cudaGetErrorString(err); return ACE_ERR_CUDA; }
    const T *Uval = (sizeof(T) == 8) ? (const T *)ctx->d_UvalD : (const T *)ctx->d_UvalF;
    dim3 g2((unsigned)((cols + 127) / 128), (unsigned)std::min<int64_t>(ctx->nB, 65535));
    if (DB)
      udb_kernel<T><<<g2, 128, 0, st>>>(cols, d.jbase, cols, ctx->nB, ctx->d_Uptr, ctx->d_Uidx, Uval,
                                         (const T *)ctx->d_scratch, out);
    else
      ub_kernel<T><<<g2, 128, 0, st>>>(ne, e0, ne, ctx->nB, ctx->d_Uptr, ctx->d_Uidx, Uval,
                                        (const T *)ctx->d_scratch, out);
    ctx->launches += 1;
    err = cudaGetLastError();
    if (err != cudaSuccess) { ctx->err = cudaGetErrorString(err); return ACE_ERR_CUDA; }
    e0 = e1;
  }
  return ACE_OK;
}

// dB for host-known offsets (off_h: host copy of the offsets)
int launch_dbasis(ace_ctx *ctx, int64_t nEnv, const int64_t *off_d, const int64_t *off_h, const double *rr,
                  const int32_t *sp, double *dB, cudaStream_t st) {
  if (nEnv == 0) return ACE_OK;
  if (ctx->prec == ACE_PREC_FP32 || ctx->prec == ACE_PREC_FP32_BF16X3)
    return run_daa<float, true>(ctx, nEnv, off_d, off_h, rr, sp, nullptr, dB, st);
  return run_daa<double, true>(ctx, nEnv, off_d, off_h, rr, sp, nullptr, dB, st);
}

int launch_adjoint_eval_d(ace_ctx *ctx, int64_t nEnv, const int64_t *off_d, const int64_t *off_h,
                          const double *rr, const int32_t *sp, const double *w, double *out, cudaStream_t st) {
  if (nEnv == 0) return ACE_OK;
  if (ctx->prec == ACE_PREC_FP32 || ctx->prec == ACE_PREC_FP32_BF16X3)
    return run_daa<float, false>(ctx, nEnv, off_d, off_h, rr, sp, w, out, st);
  return run_daa<double, false>(ctx, nEnv, off_d, off_h, rr, sp, w, out, st);
}

}  // namespace ace
