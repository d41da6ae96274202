// ace_kernels.cuh -- evaluation kernels of libace_b200.
//
// ef_kernel<TE, TG, K, NT, GRAD>: one CTA per environment (grid-stride).
//   phase 1  A_i = sum_j [mu_j == mu_i] R_{n_i}(r_j) Y_{l_i m_i}(rhat_j) in the
//            energy type TE: neighbours are staged CH at a time, one thread per
//            neighbour builds R and Y in a shared-memory slab, then one thread
//            per A entry accumulates (src/product_1pbasis.jl:99-134).
//   phase 2  the correlation functions in schedule order (ace_sched.h): each
//            thread walks a contiguous range with the current prefix path in
//            registers -- prefix products bar_d (adjoint type TG) and Horner
//            sums H_d (TE).  Closing a node of depth d folds
//            H_{d-1} += A_{v_d} H_d (energy, src/evaluator.jl:121-147) and adds
//            bar_{d-1} H_d to dAco_{v_d} (the adjoint of src/evaluator.jl:
//            174-185 / _AA_local_adjoints!, src/pibasis.jl:338-390).  Adjoint
//            targets below NPRIV go to thread-private shared-memory bins
//            (conflict free, no atomics), the rest to shared atomics.
//   phase 3  g_j = sum_i Re(dAco_i (R'_{n_i} rhat_j Y_i + R_{n_i} grad Y_i)) in
//            TG with R', grad Y recomputed per neighbour (src/evaluator.jl:187-192).
//
// aa_kernel<TE>: phase 1, then real(AA_k) written to a scratch matrix for the
//   symmetric-basis path B = U AA (src/symmbasis.jl:297-316).
#pragma once
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <type_traits>

#include "../../include/ace_b200.h"
#include "ace_arith.cuh"
#include "ace_ctx.h"
#include "ace_phi.cuh"
#include "ace_sched.h"

namespace ace {

__host__ __device__ inline size_t al16(size_t x) { return (x + 15) & ~size_t(15); }

// items per thread and iteration in the item-schedule correlation phase
#ifndef EF_ITEM_ILP
#define EF_ITEM_ILP 2
#endif
// minimum resident CTAs per SM requested from the register allocator
// (EF_MIN_BLOCKS > 0 overrides the per-type default of ef_min_blocks).
// Measured on GB300, order 4 / degree 12: the double-float kernel takes 116
// registers unconstrained (4 CTAs per SM, 2.73M env/s) and 96 at 5 (2.97M);
// FP32 and FP64 run best unconstrained (72 and 120-124 registers), which 7
// and 4 reproduce.  An explicit 1 lets the allocator take 150-210 registers
// and costs a third of the throughput.
#ifndef EF_MIN_BLOCKS
#define EF_MIN_BLOCKS 0
#endif

struct EFArgs {
  int64_t nEnv;
  const int64_t *off;
  const double *rr;
  const int32_t *sp;
  double *E;
  double *G;
  const void *tabE, *tabG;
  int ntab, nR, L, pl, pr, tp;
  // radial channels held per neighbour in the slabs: nR for the polynomial
  // basis, K (L+1) for the learned radial form, whose values come from Rext
  // ([nNbr][2 nRs]: R then dR/dr, written by the radial MLP) instead of the
  // recursion; GR ([nNbr][nRs], optional) receives dE/dR_n(r_j)
  int nRs;
  const float *Rext;
  float *GR;
  const int16_t *an, *aiy, *amu;
  int nA, nspecies;
  // correlation schedule: interleaved records and coefficients (ace_sched.h)
  const uint4 *srec;
  const void *sc;
  int64_t slen;
  // item schedule (ace_sched.h): records and (G+1) coefficient rows
  const uint4 *irec;
  const void *ic;
  int64_t in;
  double c0;
  int chunkE, chunkG, npriv;
  // task schedule (ace_sched.h build_tasks): records, (G+1) coefficient rows
  // per record row, and each warp's rows [twrow[w], twrow[w+1])
  const uint4 *trec;
  const void *tc;
  int32_t twrow[5];
  int *status;
  // compensated form: est[e] (if set) receives the environment's energy
  // rounding scale sqrt(sum_g S_g^2) 2^-24, S_g the sum of |products| that
  // share a rounding (a task of the task schedule, an item of the item runs)
  float *est;
  // environment list (if set): the launch evaluates environments
  // elist[0 .. *ecount) of the batch instead of 0 .. nEnv
  const int64_t *elist;
  const int32_t *ecount;
  // aa_kernel output
  void *AAout;
  int64_t ldE;
  const uint8_t *ord;
  const uint16_t *idx;
  int64_t nAA;
};

struct EFLayout {
  size_t tabE, tabG, an, aiy, amu, AE, AG, D, priv, pos, spc, slab, red, total;
  int slabE, slabG;
};

// comp: the compensated form keeps A as two FP32 arrays, A_hi (the adjoint's
// and the products' copy, AG) and A_lo, in the AE region (no separate AG)
inline __host__ __device__ EFLayout ef_layout(int ntab, int nR, int L, int nA, int chunkE, int chunkG,
                                              int npriv, int nt, int sE, int sG, bool same, bool radj = false,
                                              bool comp = false) {
  EFLayout l;
  size_t o = 0;
  const int szP = size_p(L), nY = size_y(L);
  l.tabE = o; o = al16(o + (size_t)ntab * sE);
  l.tabG = same ? l.tabE : o; if (!same) o = al16(o + (size_t)ntab * sG);
  l.an = o; o = al16(o + (size_t)nA * 2);
  l.aiy = o; o = al16(o + (size_t)nA * 2);
  l.amu = o; o = al16(o + (size_t)nA * 2);
  l.AE = o; o = al16(o + (size_t)nA * 2 * sE);
  l.AG = (same || comp) ? l.AE : o; if (!same && !comp) o = al16(o + (size_t)nA * 2 * sG);
  l.D = o; o = al16(o + (size_t)nA * 2 * sG);
  const int ch = chunkE > chunkG ? chunkE : chunkG;
  l.pos = o; o = al16(o + (size_t)ch * 4 * sG);
  l.spc = o; o = al16(o + (size_t)ch * 4);
  l.slabE = nR + 2 * nY;          // R, Y
  l.slabG = 2 * nR + 8 * nY + (radj ? nR : 0);  // R, dR, Y, dY [, dE/dR accumulators]
  // the neighbour slabs (phases 1, 3) and the private adjoint bins (phase 2)
  // are never live at the same time and share one region
  const size_t bE = (size_t)chunkE * l.slabE * sE, bG = (size_t)chunkG * l.slabG * sG;
  const size_t bP = (size_t)npriv * nt * 2 * sG;
  size_t big = bE > bG ? bE : bG;
  big = big > bP ? big : bP;
  l.slab = o; l.priv = o; o = al16(o + big);
  l.red = o; o = al16(o + 32 * 8);
  l.total = o;
  return l;
}

// schedule coefficients and records are read-only for a launch: loaded
// through the non-coherent read-only path
template <typename T> __device__ __forceinline__ T load_coef(const void *p, int64_t i);
template <> __device__ __forceinline__ float load_coef<float>(const void *p, int64_t i) { return __ldg((const float *)p + i); }
template <> __device__ __forceinline__ double load_coef<double>(const void *p, int64_t i) {
  return __ldg((const double *)p + i);
}
template <> __device__ __forceinline__ df load_coef<df>(const void *p, int64_t i) {
  const float2 v = __ldg((const float2 *)p + i);
  return {v.x, v.y};
}

template <typename T> __device__ __forceinline__ T load_table(const void *p, int i);
template <> __device__ __forceinline__ float load_table<float>(const void *p, int i) { return ((const float *)p)[i]; }
template <> __device__ __forceinline__ double load_table<double>(const void *p, int i) { return ((const double *)p)[i]; }
template <> __device__ __forceinline__ df load_table<df>(const void *p, int i) {
  const float2 v = ((const float2 *)p)[i];
  return {v.x, v.y};
}

// two block sums at once (blocks of at most 16 warps); valid in thread 0
__device__ __forceinline__ void block_sum2(double &v, double &u, double *red) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    v += __shfl_xor_sync(0xffffffffu, v, o);
    u += __shfl_xor_sync(0xffffffffu, u, o);
  }
  if (lane == 0) { red[w] = v; red[16 + w] = u; }
  __syncthreads();
  if (w == 0) {
    v = lane < nw ? red[lane] : 0.0;
    u = lane < nw ? red[16 + lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      v += __shfl_xor_sync(0xffffffffu, v, o);
      u += __shfl_xor_sync(0xffffffffu, u, o);
    }
  }
  __syncthreads();
}

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

// Phase 1: A (type T) for the environment's neighbours rr[o0 .. o0+J).
// Neighbours are staged `chunk` at a time; thread (jj, m) = (t / (L+1),
// t % (L+1)) evaluates column m of Y for neighbour jj (and R_n when m == 0),
// then one thread per A entry accumulates.  Requires chunk * (L+1) <= blockDim.
// SPLIT (T = df): A is stored as two FP32 arrays, A_hi = ((cpx<float> *)A)[i]
// and A_lo = ((cpx<float> *)A)[nA + i], instead of nA double-float pairs.
template <typename T, bool SPLIT>
__device__ __forceinline__ cpx<T> a_load(const cpx<T> *A, int nA, int i) {
  if constexpr (SPLIT) {
    const cpx<float> h = ((const cpx<float> *)A)[i], l = ((const cpx<float> *)A)[nA + i];
    return {Arith<T>::from_pair(h.re, l.re), Arith<T>::from_pair(h.im, l.im)};
  } else {
    return A[i];
  }
}
template <typename T, bool SPLIT>
__device__ __forceinline__ void a_store(cpx<T> *A, int nA, int i, cpx<T> v) {
  if constexpr (SPLIT) {
    ((cpx<float> *)A)[i] = {Arith<T>::hi(v.re), Arith<T>::hi(v.im)};
    ((cpx<float> *)A)[nA + i] = {Arith<T>::lo(v.re), Arith<T>::lo(v.im)};
  } else {
    A[i] = v;
  }
}

template <typename T, bool SPLIT = false>
__device__ __forceinline__ void build_A(const EFArgs &a, const Tables<T> &tb, int64_t o0, int J, int chunk,
                                        int SE, const int16_t *s_an, const int16_t *s_aiy, const int16_t *s_amu,
                                        int *ssp, T *slab, cpx<T> *A) {
  static_assert(!SPLIT || std::is_same<T, df>::value, "split storage holds double-float values");
  const int tid = threadIdx.x, nt = blockDim.x;
  const int LP1 = a.L + 1;
  const int jj = tid / LP1, m = tid - jj * LP1;
  for (int i = tid; i < a.nA; i += nt) a_store<T, SPLIT>(A, a.nA, i, {Arith<T>::zero(), Arith<T>::zero()});
  for (int c0 = 0; c0 < J; c0 += chunk) {
    const int nc = min(chunk, J - c0);
    __syncthreads();
    if (jj < nc) {
      const int64_t j = o0 + c0 + jj;
      const double xd = a.rr[3 * j], yd = a.rr[3 * j + 1], zd = a.rr[3 * j + 2];
      const T x = Arith<T>::from(xd), y = Arith<T>::from(yd), z = Arith<T>::from(zd);
      const Angles<T> g = angles(x, y, z);
      T *sl = slab + (size_t)jj * SE;
      if (m == 0) {
        int s = 0;
        if (a.nspecies > 1) {
          s = a.sp[j];
          if (s < 0 || s >= a.nspecies) { atomicOr(a.status, ACE_STATUS_BAD_SPECIES); s = -1; }
        }
        ssp[jj] = s;
        const double rd = sqrt(xd * xd + yd * yd + zd * zd);
        if (!(rd > 0.0) || !isfinite(rd)) atomicOr(a.status, ACE_STATUS_BAD_POSITION);
        if (!a.Rext) radial_eval<T, false>(tb, g.r, sl, nullptr);
      }
      if (a.Rext)
        for (int n = m; n < a.nRs; n += LP1) sl[n] = Arith<T>::from((double)a.Rext[(size_t)j * 2 * a.nRs + n]);
      sh_col_values<T>(tb, g, m, (cpx<T> *)(sl + a.nRs));
    }
    __syncthreads();
    for (int i = tid; i < a.nA; i += nt) {
      const int n = s_an[i], iy = s_aiy[i], mu = s_amu[i];
      cpx<T> acc = a_load<T, SPLIT>(A, a.nA, i);
      for (int q = 0; q < nc; ++q) {
        if (a.nspecies > 1 && ssp[q] != mu) continue;
        const T *sl = slab + (size_t)q * SE;
        const cpx<T> Y = ((const cpx<T> *)(sl + a.nRs))[iy];
        acc = cfma(acc, Y, sl[n]);
      }
      a_store<T, SPLIT>(A, a.nA, i, acc);
    }
  }
  __syncthreads();
}

// Re(a b)
template <typename T> __device__ __forceinline__ T re_mul(cpx<T> a, cpx<T> b) { return a.re * b.re - a.im * b.im; }
#if ACE_DF_DOT2
template <> __device__ __forceinline__ df re_mul<df>(cpx<df> a, cpx<df> b) { return dot2(a.re, b.re, -a.im, b.im); }
#endif

template <typename T> __device__ __forceinline__ cpx<T> shfl_down_c(cpx<T> v, int off) {
  return {__shfl_down_sync(0xffffffffu, v.re, off), __shfl_down_sync(0xffffffffu, v.im, off)};
}

// ITEMS selects the phase-2 algorithm: false = per-thread trie walk over the
// lexicographic schedule, true = uniform items (ace_sched.h build_items).
// CPX (item schedule only): complex coefficients c = (re, im), stored as
// (G+1) rows of real parts followed by (G+1) rows of imaginary parts; the
// output is Re(sum_k c_k AA_k) (the Cartesian components of an
// EuclideanVector model).
template <typename TE, int K> constexpr int ef_min_blocks() {
  return EF_MIN_BLOCKS > 0 ? EF_MIN_BLOCKS
         : K <= 4 ? (std::is_same<TE, df>::value ? 5 : std::is_same<TE, double>::value ? 4 : 7)
                  : (std::is_same<TE, df>::value ? 4 : std::is_same<TE, double>::value ? 3 : 5);
}
// COMP (compensated form; TE = df, TG = float, item schedule): A is built in
// double-float as in the fp32x2 form, but the correlation products run in
// FP32 on A_hi = the FP32 rounding of A, with FP32 coefficients, and each
// item's energy term is added to a double-float accumulator.  The rounding
// A_lo = A - A_hi is put back to first order after the adjoint pass:
// E = E(A_hi) + Re sum_i dE/dA_i(A_hi) A_lo_i, the adjoint being the one the
// forces need anyway.  The remaining error is the FP32 rounding of the
// products, which does not add coherently over the terms.
// resident CTAs per SM of the compensated form: FP32 item state plus the
// double-float A build and energy accumulator (no spills at orders 2-5)
template <int K> constexpr int comp_min_blocks() { return EF_MIN_BLOCKS > 0 ? EF_MIN_BLOCKS : K <= 4 ? 6 : K == 5 ? 5 : 4; }
// TASKS (item family, orders >= 3, NT = 128): the correlation phase walks the
// task schedule (ace_sched.h build_tasks) instead of the per-thread item runs.
// MINB > 0 overrides the resident CTAs per SM requested from the register
// allocator (the task-schedule kernels keep little state per thread and have
// a second, high-occupancy instantiation the autotuner can pick).
template <typename TE, typename TG, int K, int NT, bool GRAD, bool ITEMS, bool CPX = false, bool COMP = false,
          bool TASKS = false, int MINB = 0>
__global__ void __launch_bounds__(NT, MINB > 0 ? MINB
                                      : COMP ? comp_min_blocks<K>() : ef_min_blocks<TE, CPX ? K + 1 : K>())
    ef_kernel(EFArgs a) {
  static_assert(ITEMS || !CPX, "complex coefficients need the item schedule");
  static_assert(!TASKS || (ITEMS && !CPX && K >= 3 && NT == 128), "the task schedule: real coefficients, K >= 3");
  static_assert(!COMP || (ITEMS && GRAD && !CPX && (EF_ITEM_RUNS || TASKS) && std::is_same<TE, df>::value &&
                          std::is_same<TG, float>::value),
                "the compensated form is the double-float A with FP32 item products and the run adjoint");
  constexpr bool SAME = std::is_same<TE, TG>::value;
  // arithmetic type of the correlation products
  using TL = std::conditional_t<COMP, float, TE>;
  extern __shared__ __align__(16) unsigned char sm[];
  const EFLayout lay = ef_layout(a.ntab, a.nRs, a.L, a.nA, a.chunkE, a.chunkG, a.npriv, NT, sizeof(TE),
                                 sizeof(TG), SAME, a.Rext != nullptr, COMP);
  TE *tabE = (TE *)(sm + lay.tabE);
  TG *tabG = (TG *)(sm + lay.tabG);
  int16_t *s_an = (int16_t *)(sm + lay.an);
  int16_t *s_aiy = (int16_t *)(sm + lay.aiy);
  int16_t *s_amu = (int16_t *)(sm + lay.amu);
  cpx<TE> *AE = (cpx<TE> *)(sm + lay.AE);
  cpx<TG> *AG = (cpx<TG> *)(sm + lay.AG);
  cpx<TG> *D = (cpx<TG> *)(sm + lay.D);
  cpx<TG> *priv = (cpx<TG> *)(sm + lay.priv);
  TG *spos = (TG *)(sm + lay.pos);
  int *ssp = (int *)(sm + lay.spc);
  double *red = (double *)(sm + lay.red);
  const int tid = threadIdx.x;
  const int nY = size_y(a.L);
  const int npriv = a.npriv;

  for (int i = tid; i < a.ntab; i += NT) {
    tabE[i] = load_table<TE>(a.tabE, i);
    if (!SAME) tabG[i] = load_table<TG>(a.tabG, i);
  }
  for (int i = tid; i < a.nA; i += NT) { s_an[i] = a.an[i]; s_aiy[i] = a.aiy[i]; s_amu[i] = a.amu[i]; }
  __syncthreads();
  Tables<TE> tbE;
  tbE.bind(tabE, a.nR, a.L, a.pl, a.pr, a.tp);
  Tables<TG> tbG;
  tbG.bind(tabG, a.nR, a.L, a.pl, a.pr, a.tp);
  const int64_t ntot = a.off[a.nEnv];
  const int64_t nrun = a.elist ? (int64_t)*a.ecount : a.nEnv;

  for (int64_t q = blockIdx.x; q < nrun; q += gridDim.x) {
    const int64_t e = a.elist ? a.elist[q] : q;
    const int64_t o0 = a.off[e], o1 = a.off[e + 1];
    if (o0 < 0 || o1 < o0 || o1 > ntot) {
      if (tid == 0) {
        atomicOr(a.status, ACE_STATUS_BAD_OFFSETS);
        a.E[e] = __longlong_as_double(0x7ff8000000000000ll);
      }
      continue;
    }
    const int J = (int)(o1 - o0);
    // ---------------- phase 1
    build_A<TE, COMP>(a, tbE, o0, J, a.chunkE, lay.slabE, s_an, s_aiy, s_amu, ssp, (TE *)(sm + lay.slab), AE);
    if (GRAD) {
      for (int i = tid; i < a.nA; i += NT) {
        // (the compensated form's A_hi already is the adjoint's copy)
        if (!SAME && !COMP) AG[i] = {lower<TG>(AE[i].re), lower<TG>(AE[i].im)};
        D[i] = {TG(0), TG(0)};
      }
      for (int i = tid; i < npriv * NT; i += NT) priv[i] = {TG(0), TG(0)};
      __syncthreads();
    }
    // ---------------- phase 2
    auto dacc = [&](int u, cpx<TG> v) {
      if (u < npriv) {
        cpx<TG> *p = priv + u * NT + tid;
        p->re += v.re;
        p->im += v.im;
      } else {
        atomicAdd(&D[u].re, v.re);
        atomicAdd(&D[u].im, v.im);
      }
    };
    TE eacc = Arith<TE>::zero();
    float est2 = 0.0f;  // compensated form: sum of squared rounding groups
    // the correlation phase reads A in its own arithmetic type
    const cpx<TL> *AL;
    if constexpr (COMP) AL = (const cpx<TL> *)AG; else AL = (const cpx<TL> *)AE;
    if constexpr (!ITEMS) {
    cpx<TE> H[K + 1], Ac[K + 1];
    cpx<TG> bar[K + 1];
    int vc[K + 1];
#pragma unroll
    for (int d = 0; d <= K; ++d) {
      H[d] = {Arith<TE>::zero(), Arith<TE>::zero()};
      Ac[d] = H[d];
      bar[d] = {TG(1), TG(0)};
      vc[d] = 0;
    }
    int cur = 0;
    auto close = [&](int d) {
      if (d == K) {  // leaf: H_K is the (real) coefficient
        if (GRAD) dacc(vc[K], cscale(bar[K - 1], lower<TG>(H[K].re)));
        H[K - 1] = cadd(H[K - 1], cscale(Ac[K], H[K].re));
      } else {
        if (GRAD) dacc(vc[d], cmul(bar[d - 1], cpx<TG>{lower<TG>(H[d].re), lower<TG>(H[d].im)}));
        H[d - 1] = cadd(H[d - 1], cmul(Ac[d], H[d]));
      }
    };
    for (int64_t j = 0; j < a.slen; ++j) {
      const int64_t slot = j * NT + tid;
      const uint4 rc = a.srec[slot];
      const int k = rc.w & 0xff, q = (rc.w >> 8) & 0xff;
      if (k == 0) continue;
      const TE c = load_coef<TE>(a.sc, slot);
      const uint32_t vw[3] = {rc.x, rc.y, rc.z};
#pragma unroll
      for (int d = K; d >= 1; --d)
        if (d <= cur && d > q) close(d);
#pragma unroll
      for (int d = 1; d <= K; ++d) {
        if (d > q && d <= k) {
          const int u = (vw[(d - 1) >> 1] >> (16 * ((d - 1) & 1))) & 0xffff;
          vc[d] = u;
          Ac[d] = AE[u];
          if (GRAD && d < K) bar[d] = cmul(bar[d - 1], AG[u]);
          H[d] = {Arith<TE>::zero(), Arith<TE>::zero()};
        }
      }
#pragma unroll
      for (int d = 1; d <= K; ++d)
        if (d == k) H[d].re = H[d].re + c;
      cur = k;
    }
#pragma unroll
    for (int d = K; d >= 1; --d)
      if (d <= cur) close(d);
      eacc = H[0].re;
    } else if constexpr (TASKS) {
      // Each warp runs its rows of the task schedule; a row is uniform
      // across the warp (one type, one item count), so the lanes run their
      // tasks in lockstep.  Per task: Q_t = prod A_t; per item Q = Q_t A_mid,
      // the energy Re(Q H), H = c_own + sum_g c_g A_leaf_g, and the
      // adjoints D[leaf_g] += Q c_g, D[mid] += H Q_t, W += H A_mid; at the
      // end D[t_d] += W prod_{d' != d} A_t_d'.  Short items: the flat
      // product and its local adjoints.
      constexpr int KT = (K >= 3) ? K - 2 : 1;
      constexpr int G1 = ITEM_G + 1;
      constexpr bool ONE = std::is_same<TL, TG>::value;  // products and adjoint in one type
      const int lane = tid & 31, wp = tid >> 5;
      const cpx<TG> gone = {TG(1), TG(0)};
      const TL ze = Arith<TL>::zero();
      // the next row's record (header, item) is loaded one step ahead, so
      // its L2 latency overlaps the current step's arithmetic
      const int64_t rend = a.twrow[wp + 1];
      auto load_item = [&](int64_t ir, uint4 &rc, TL &c0, TL (&cg)[ITEM_G]) __attribute__((always_inline)) {
        rc = __ldg(a.trec + ir * 32 + lane);
        const int64_t cb = ir * (G1 * 32) + lane;
        c0 = load_coef<TL>(a.tc, cb);
#pragma unroll
        for (int g = 0; g < ITEM_G; ++g) cg[g] = load_coef<TL>(a.tc, cb + (g + 1) * 32);
      };
      int64_t row = a.twrow[wp];
      uint4 hr = row < rend ? __ldg(a.trec + row * 32 + lane) : make_uint4(0u, 0u, 0u, 0u);
      while (row < rend) {
        const int type = (int)(hr.w >> 16), n = (int)(hr.w & 0xffffu);
        const uint32_t hw[2] = {hr.x, hr.y};
        const int64_t next = row + 1 + (type == 1 ? n : 0);
        const uint4 hnext = next < rend ? __ldg(a.trec + next * 32 + lane) : make_uint4(0u, 0u, 0u, 0u);
        if (type == 1) {
          int t[KT];
          cpx<TG> ag[KT];
          cpx<TL> QtL = {Arith<TL>::one(), ze};
#pragma unroll
          for (int d = 0; d < KT; ++d) {
            t[d] = (int)((hw[d >> 1] >> (16 * (d & 1))) & 0xffffu);
            const cpx<TL> av = AL[t[d]];
            QtL = (d == 0) ? av : cmul(QtL, av);
            ag[d] = {lower<TG>(av.re), lower<TG>(av.im)};
          }
          cpx<TG> QtG = gone;
          if constexpr (ONE) {
            QtG = {lower<TG>(QtL.re), lower<TG>(QtL.im)};
          } else {
#pragma unroll
            for (int d = 0; d < KT; ++d) QtG = (d == 0) ? ag[d] : cmul(QtG, ag[d]);
          }
          cpx<TG> Wt = {TG(0), TG(0)};
          float eterm = 0.0f;  // compensated form: the task's energy terms
          float esz = 0.0f;    // and the sum of their products' magnitudes
          uint4 rcn = make_uint4(0u, 0u, 0u, 0u);
          TL c0n = ze, cgn[ITEM_G];
#pragma unroll
          for (int g = 0; g < ITEM_G; ++g) cgn[g] = ze;
          if (n > 0) load_item(row + 1, rcn, c0n, cgn);
          for (int j = 0; j < n; ++j) {
            const uint4 rc = rcn;
            TL cg[ITEM_G];
#pragma unroll
            for (int g = 0; g < ITEM_G; ++g) cg[g] = cgn[g];
            cpx<TL> H = {c0n, ze};
            if (j + 1 < n) load_item(row + 2 + j, rcn, c0n, cgn);
            const int mid = (int)(rc.x & 0xffffu), nl = (int)(rc.w & 0xffffu);
            const int lf[2] = {(int)(rc.x >> 16), (int)(rc.y & 0xffffu)};
#pragma unroll
            for (int g = 0; g < ITEM_G; ++g)
              if (g < nl) H = cfma(H, AL[lf[g < 2 ? g : 0]], cg[g]);
            const cpx<TL> am = AL[mid];
            const cpx<TL> QL = cmul(QtL, am);
            if constexpr (COMP) {
              const float p1 = QL.re * H.re, p2 = QL.im * H.im;
              eterm += p1 - p2;
              esz += fabsf(p1) + fabsf(p2);
            } else {
              eacc = eacc + re_mul<TE>(QL, H);
            }
            if (GRAD) {
              const cpx<TG> amg = {lower<TG>(am.re), lower<TG>(am.im)};
              cpx<TG> QG;
              if constexpr (ONE) QG = {lower<TG>(QL.re), lower<TG>(QL.im)};
              else QG = cmul(QtG, amg);
              const cpx<TG> h = {lower<TG>(H.re), lower<TG>(H.im)};
#pragma unroll
              for (int g = 0; g < ITEM_G; ++g)
                if (g < nl) dacc(lf[g < 2 ? g : 0], cscale(QG, lower<TG>(cg[g])));
              dacc(mid, cmul(h, QtG));
              Wt = cadd(Wt, cmul(h, amg));
            }
          }
          if constexpr (COMP) {
            eacc = eacc + df{eterm, 0.0f};
            est2 = fmaf(esz, esz, est2);
          }
          if (GRAD) {
            // W over the task prefix: prefix and suffix products
            cpx<TG> pre = gone;
#pragma unroll
            for (int d = 0; d < KT; ++d) {
              cpx<TG> suf = gone;
#pragma unroll
              for (int e = d + 1; e < KT; ++e) suf = (e == d + 1) ? ag[e] : cmul(suf, ag[e]);
              dacc(t[d], cmul(Wt, cmul(pre, suf)));
              pre = (d == 0) ? ag[0] : cmul(pre, ag[d]);
            }
          }
        } else {
          // short item: P = n < K - 1 indices in [0..P)
          const int P = n;
          const TL c = load_coef<TL>(a.tc, row * (G1 * 32) + lane);
          int v[KT];
          cpx<TG> ag[KT];
          cpx<TL> p = {Arith<TL>::one(), ze};
#pragma unroll
          for (int d = 0; d < KT; ++d) {
            v[d] = (int)((hw[d >> 1] >> (16 * (d & 1))) & 0xffffu);
            ag[d] = gone;
            if (d < P) {
              const cpx<TL> av = AL[v[d]];
              p = (d == 0) ? av : cmul(p, av);
              ag[d] = {lower<TG>(av.re), lower<TG>(av.im)};
            }
          }
          if constexpr (COMP) {
            const float t = c * p.re;
            eacc = eacc + df{t, 0.0f};
            est2 = fmaf(t, t, est2);
          } else {
            eacc = eacc + c * p.re;
          }
          if (GRAD) {
            const TG cG = lower<TG>(c);
            cpx<TG> pre = gone;
#pragma unroll
            for (int d = 0; d < KT; ++d) {
              if (d < P) {
                cpx<TG> suf = gone;
#pragma unroll
                for (int e = d + 1; e < KT; ++e)
                  if (e < P) suf = cmul(suf, ag[e]);
                dacc(v[d], cscale(cmul(pre, suf), cG));
                pre = cmul(pre, ag[d]);
              }
            }
          }
        }
        row = next;
        hr = hnext;
      }
    } else {
      // EF_ITEM_ILP items per thread and iteration, interleaved: their
      // product chains and warp reductions are independent, which hides the
      // latency of the dependent double-float arithmetic
      constexpr int KP = (K > 1) ? K - 1 : 1;
      constexpr int IU = EF_ITEM_ILP;
#if !EF_ITEM_RUNS
      const int lane = tid & 31;
#endif
      const cpx<TG> gone = {TG(1), TG(0)};
      const TL ze = Arith<TL>::zero();
#if EF_ITEM_RUNS
      // reverse-mode accumulation along this thread's run of items (sorted
      // by prefix): the open path cur[0..cP) of the prefix trie with, per
      // depth d, A at that node (acur), the product Q[d] = A_cur[0] ..
      // A_cur[d] and the node's adjoint W[d] = dE/dQ[d].  A node closes when
      // the path leaves it: D[cur[d]] += W[d] Q[d-1] and W[d-1] += W[d] acur[d]
      // (the same sums as the per-item products over the other prefix
      // members, src/pibasis.jl:338-390, grouped by trie node)
      int cur[KP], cP = 0;
      cpx<TG> W[KP], Q[KP], acur[KP];
#pragma unroll
      for (int d = 0; d < KP; ++d) { cur[d] = -1; W[d] = {TG(0), TG(0)}; Q[d] = gone; acur[d] = gone; }
      auto close_to = [&](int c) __attribute__((always_inline)) {
#pragma unroll
        for (int d = KP - 1; d >= 0; --d) {
          const bool cl = d >= c && d < cP;
          const int dm = d > 0 ? d - 1 : 0;
          const cpx<TG> w = W[d];
          if (cl) dacc(cur[d], d > 0 ? cmul(w, Q[dm]) : w);
          if (d > 0) {
            const cpx<TG> t = cmul(w, acur[d]);
            W[dm].re += cl ? t.re : TG(0);
            W[dm].im += cl ? t.im : TG(0);
          }
          W[d].re = cl ? TG(0) : w.re;
          W[d].im = cl ? TG(0) : w.im;
        }
      };
#endif
      for (int64_t f0 = tid; f0 < a.in; f0 += (int64_t)IU * NT) {
        int P[IU], nl[IU], vi[IU][KP], ul[IU][ITEM_G];
        unsigned heads[IU];
        cpx<TL> bar[IU], H[IU];
        cpx<TG> aG[IU][KP];
        TL cl[IU][ITEM_G], cli[IU][ITEM_G];
#pragma unroll
        for (int u = 0; u < IU; ++u) {
          const int64_t f = f0 + (int64_t)u * NT;
          // item_n is a multiple of NT, so `ok` is uniform across the CTA
          const bool ok = f < a.in;
          const uint4 rc = ok ? __ldg(a.irec + f) : make_uint4(0u, 0u, 0u, 0u);
          P[u] = (rc.w >> 16) & 0xf;
          nl[u] = (rc.w >> 20) & 0xf;
          heads[u] = (rc.w >> 24) & 0xff;
          const uint32_t vw[4] = {rc.x, rc.y, rc.z, rc.w};
          bar[u] = {Arith<TL>::one(), ze};
#pragma unroll
          for (int d = 0; d < KP; ++d) {
            vi[u][d] = (int)((vw[d >> 1] >> (16 * (d & 1))) & 0xffff);
            aG[u][d] = gone;
            if (d < P[u]) {
              const cpx<TL> ae = AL[vi[u][d]];
              // (the compensated form takes the prefix product from the
              // adjoint's path products Q below instead)
              if constexpr (!COMP) bar[u] = (d == 0) ? ae : cmul(bar[u], ae);
              // the adjoint's copy of A (AG = lower(AE)) from the value in registers
              if (GRAD) aG[u][d] = {lower<TG>(ae.re), lower<TG>(ae.im)};
            }
          }
          H[u] = {ok ? load_coef<TL>(a.ic, f) : ze, (CPX && ok) ? load_coef<TL>(a.ic, (int64_t)(ITEM_G + 1) * a.in + f) : ze};
#pragma unroll
          for (int g = 0; g < ITEM_G; ++g) {
            ul[u][g] = (int)((vw[(5 + g) >> 1] >> (16 * ((5 + g) & 1))) & 0xffff);
            cl[u][g] = ok ? load_coef<TL>(a.ic, (int64_t)(g + 1) * a.in + f) : ze;
            cli[u][g] = (CPX && ok) ? load_coef<TL>(a.ic, (int64_t)(ITEM_G + 2 + g) * a.in + f) : ze;
            if (g < nl[u]) {
              if constexpr (CPX) H[u] = cadd(H[u], cmul(AL[ul[u][g]], cpx<TL>{cl[u][g], cli[u][g]}));
              else H[u] = cfma(H[u], AL[ul[u][g]], cl[u][g]);
            }
          }
        }
        if constexpr (!COMP) {
#pragma unroll
          for (int u = 0; u < IU; ++u)
            if (P[u] > 0) eacc = eacc + re_mul<TE>(bar[u], H[u]);
        }
        if (GRAD) {
#if EF_ITEM_RUNS
          float eterm = 0.0f;  // compensated form: this iteration's energy terms
#pragma unroll
          for (int u = 0; u < IU; ++u) {
            if (P[u] > 0) {
              const cpx<TG> h = {lower<TG>(H[u].re), lower<TG>(H[u].im)};
              // depth of the first difference between the item's prefix and the path
              int c = 0;
#pragma unroll
              for (int d = 0; d < KP; ++d)
                if (c == d && d < P[u] && d < cP && vi[u][d] == cur[d]) c = d + 1;
              close_to(c);
              // extend the path by the item's prefix below depth c
#pragma unroll
              for (int d = 0; d < KP; ++d) {
                const bool ext = d >= c && d < P[u];
                const cpx<TG> q = d > 0 ? cmul(Q[d > 0 ? d - 1 : 0], aG[u][d]) : aG[u][d];
                cur[d] = ext ? vi[u][d] : cur[d];
                acur[d] = ext ? aG[u][d] : acur[d];
                Q[d] = ext ? q : Q[d];
              }
              cP = P[u];
#pragma unroll
              for (int d = 0; d < KP; ++d) {
                // selects, not a branch: keeps W in registers
                const bool leaf = d == cP - 1;
                W[d].re += leaf ? h.re : TG(0);
                W[d].im += leaf ? h.im : TG(0);
              }
              if constexpr (COMP) {
                // the item's prefix product is the path product at its depth
                // (selected, not indexed: Q stays in registers)
                cpx<TG> qd = Q[0];
#pragma unroll
                for (int d = 1; d < KP; ++d) {
                  const bool at = d == cP - 1;
                  qd.re = at ? Q[d].re : qd.re;
                  qd.im = at ? Q[d].im : qd.im;
                }
                const float p1 = qd.re * h.re, p2 = qd.im * h.im;
                eterm += p1 - p2;
                const float sz = fabsf(p1) + fabsf(p2);
                est2 = fmaf(sz, sz, est2);
              }
              // only full-length prefixes carry leaves
              const cpx<TG> bG = Q[KP - 1];
#pragma unroll
              for (int g = 0; g < ITEM_G; ++g)
                if (g < nl[u]) {
                  if constexpr (CPX) dacc(ul[u][g], cmul(bG, cpx<TG>{lower<TG>(cl[u][g]), lower<TG>(cli[u][g])}));
                  else dacc(ul[u][g], cscale(bG, lower<TG>(cl[u][g])));
                }
            }
          }
          if constexpr (COMP) eacc = eacc + df{eterm, 0.0f};
#else
          cpx<TG> v[IU][KP];
#pragma unroll
          for (int u = 0; u < IU; ++u) {
            const cpx<TG> h = {lower<TG>(H[u].re), lower<TG>(H[u].im)};
            cpx<TG> bG;
            {
              cpx<TG> pre[KP], suf[KP];
              pre[0] = gone;
#pragma unroll
              for (int d = 1; d < KP; ++d) pre[d] = (d < P[u]) ? cmul(pre[d - 1], aG[u][d - 1]) : pre[d - 1];
              suf[KP - 1] = gone;
#pragma unroll
              for (int d = KP - 2; d >= 0; --d) suf[d] = (d + 1 < P[u]) ? cmul(aG[u][d + 1], suf[d + 1]) : gone;
              bG = cmul(pre[KP - 1], aG[u][KP - 1]);
#pragma unroll
              for (int d = 0; d < KP; ++d)
                v[u][d] = (d < P[u]) ? cmul(cmul(pre[d], suf[d]), h) : cpx<TG>{TG(0), TG(0)};
            }
#pragma unroll
            for (int g = 0; g < ITEM_G; ++g)
              if (g < nl[u]) {
                if constexpr (CPX) dacc(ul[u][g], cmul(bG, cpx<TG>{lower<TG>(cl[u][g]), lower<TG>(cli[u][g])}));
                else dacc(ul[u][g], cscale(bG, lower<TG>(cl[u][g])));
              }
          }
#pragma unroll
          for (int d = 0; d < KP; ++d) {
            if (d < KP - 1) {
              // runs of equal (v1..v_{d+1}) are adjacent lanes: reduce into each run's head
              unsigned hm[IU];
#pragma unroll
              for (int u = 0; u < IU; ++u) hm[u] = __ballot_sync(0xffffffffu, (heads[u] >> d) & 1u);
#pragma unroll
              for (int off = 1; off < 32; off <<= 1) {
#pragma unroll
                for (int u = 0; u < IU; ++u) {
                  const cpx<TG> o = shfl_down_c(v[u][d], off);
                  const unsigned between =
                      (unsigned)(((unsigned long long)hm[u] >> (lane + 1)) & ((1ull << off) - 1ull));
                  if (lane + off < 32 && between == 0u) { v[u][d].re += o.re; v[u][d].im += o.im; }
                }
              }
#pragma unroll
              for (int u = 0; u < IU; ++u)
                if (((heads[u] >> d) & 1u) && d < P[u]) dacc(vi[u][d], v[u][d]);
            } else {
#pragma unroll
              for (int u = 0; u < IU; ++u)
                if (d < P[u]) dacc(vi[u][d], v[u][d]);
            }
          }
#endif
        }
      }
#if EF_ITEM_RUNS
      if (GRAD) close_to(0);
#endif
    }
    double eloc = lower<double>(eacc);
    if constexpr (!COMP) {
      const double esum = block_sum(eloc, red);
      if (tid == 0) a.E[e] = a.c0 + esum;
    }
    if (!GRAD) continue;
    // every thread's item loop has written its private bins and atomics
    // (without the energy's block sum above, the compensated form needs
    // this barrier of its own)
    if constexpr (COMP) __syncthreads();
    // private bins -> D (one warp per bin, lanes over threads)
    {
      const int lane = tid & 31, w = tid >> 5;
      for (int u = w; u < npriv; u += NT / 32) {
        TG sr = TG(0), si = TG(0);
        for (int t = lane; t < NT; t += 32) {
          const cpx<TG> *p = priv + u * NT + t;
          sr += p->re; si += p->im;
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          sr += __shfl_xor_sync(0xffffffffu, sr, o);
          si += __shfl_xor_sync(0xffffffffu, si, o);
        }
        if (lane == 0 && u < a.nA) { D[u].re += sr; D[u].im += si; }
      }
      __syncthreads();
    }
    if constexpr (COMP) {
      // first-order correction for the FP32 rounding of A: Re sum_i D_i A_lo_i
      const cpx<float> *Alo = (const cpx<float> *)AE + a.nA;
      for (int i = tid; i < a.nA; i += NT) {
        const cpx<float> lo = Alo[i];
        const cpx<TG> d = D[i];
        eloc += (double)d.re * (double)lo.re - (double)d.im * (double)lo.im;
      }
      static_assert(!COMP || NT <= 512, "block_sum2: at most 16 warps");
      double esum = eloc, esq = (double)est2;
      block_sum2(esum, esq, red);
      if (tid == 0) {
        a.E[e] = a.c0 + esum;
        if (a.est) a.est[e] = (float)(sqrt(esq) * 0x1p-24);
      }
      if (!a.G && !a.GR) continue;  // energies only
    }
    // ---------------- phase 3: forces
    const int lane = tid & 31, w = tid >> 5, nw = NT >> 5;
    TG *slab = (TG *)(sm + lay.slab);
    const int SG = lay.slabG;
    const int LP1 = a.L + 1;
    const int cj = tid / LP1, cm = tid - cj * LP1;
    for (int c0 = 0; c0 < J; c0 += a.chunkG) {
      const int nc = min(a.chunkG, J - c0);
      __syncthreads();
      if (cj < nc) {
        const int64_t j = o0 + c0 + cj;
        const TG x = TG(a.rr[3 * j]), y = TG(a.rr[3 * j + 1]), z = TG(a.rr[3 * j + 2]);
        const Angles<TG> g = angles(x, y, z);
        TG *sl = slab + (size_t)cj * SG;
        cpx<TG> *Yc = (cpx<TG> *)(sl + 2 * a.nRs);
        if (a.Rext) {
          const float *rx = a.Rext + (size_t)j * 2 * a.nRs;
          for (int n = cm; n < a.nRs; n += LP1) {
            sl[n] = TG(rx[n]);
            sl[a.nRs + n] = TG(rx[a.nRs + n]);
            sl[2 * a.nRs + 8 * nY + n] = TG(0);
          }
        }
        if (cm == 0) {
          int s = 0;
          if (a.nspecies > 1) {
            s = a.sp[j];
            if (s < 0 || s >= a.nspecies) s = -1;
          }
          ssp[cj] = s;
          spos[4 * cj + 0] = x / g.r; spos[4 * cj + 1] = y / g.r; spos[4 * cj + 2] = z / g.r;
          if (!a.Rext) radial_eval<TG, true>(tbG, g.r, sl, sl + a.nRs);
        }
        sh_col_grad<TG>(tbG, g, cm, Yc, Yc + nY);
      }
      __syncthreads();
      for (int jj = w; jj < nc; jj += nw) {
        TG *sl = slab + (size_t)jj * SG;
        const cpx<TG> *Y = (const cpx<TG> *)(sl + 2 * a.nRs);
        const cpx<TG> *dY = Y + nY;
        TG *sgr = sl + 2 * a.nRs + 8 * nY;
        const int s = ssp[jj];
        TG g0 = TG(0), g1 = TG(0), g2 = TG(0), gr = TG(0);
        for (int i = lane; i < a.nA; i += 32) {
          if (a.nspecies > 1 && s_amu[i] != s) continue;
          const int n = s_an[i], iy = s_aiy[i];
          const cpx<TG> d = D[i];
          const TG R = sl[n], dR = sl[a.nRs + n];
          const cpx<TG> y0 = Y[iy];
          const TG p = d.re * y0.re - d.im * y0.im;
          gr += dR * p;
          if (a.GR) atomicAdd(sgr + n, p);
          const cpx<TG> *dy = dY + 3 * iy;
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
        if (lane == 0 && a.G) {
          const int64_t j = o0 + c0 + jj;
          a.G[3 * j + 0] = (double)(gr * spos[4 * jj + 0] + g0);
          a.G[3 * j + 1] = (double)(gr * spos[4 * jj + 1] + g1);
          a.G[3 * j + 2] = (double)(gr * spos[4 * jj + 2] + g2);
        }
      }
      if (a.GR) {  // dE/dR_n(r_j) of the chunk, written contiguously
        __syncthreads();
        for (int q = tid; q < nc * a.nRs; q += NT) {
          const int jj = q / a.nRs, n = q - jj * a.nRs;
          a.GR[(size_t)(o0 + c0 + jj) * a.nRs + n] = (float)slab[(size_t)jj * SG + 2 * a.nRs + 8 * nY + n];
        }
      }
    }
    __syncthreads();
  }
}

// Phase 1, then real(AA_k) (flat products, src/pibasis.jl:265-275) for
// environments e0 + [0, ldE) into AAout[k * ldE + e].
template <typename TE, typename TO>
__global__ void __launch_bounds__(256) aa_kernel(EFArgs a) {
  extern __shared__ __align__(16) unsigned char sm[];
  const EFLayout lay = ef_layout(a.ntab, a.nRs, a.L, a.nA, a.chunkE, 1, 0, 256, sizeof(TE), sizeof(TE), true);
  TE *tabE = (TE *)(sm + lay.tabE);
  int16_t *s_an = (int16_t *)(sm + lay.an);
  int16_t *s_aiy = (int16_t *)(sm + lay.aiy);
  int16_t *s_amu = (int16_t *)(sm + lay.amu);
  cpx<TE> *AE = (cpx<TE> *)(sm + lay.AE);
  int *ssp = (int *)(sm + lay.spc);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < a.ntab; i += nt) tabE[i] = load_table<TE>(a.tabE, i);
  for (int i = tid; i < a.nA; i += nt) { s_an[i] = a.an[i]; s_aiy[i] = a.aiy[i]; s_amu[i] = a.amu[i]; }
  __syncthreads();
  Tables<TE> tb;
  tb.bind(tabE, a.nR, a.L, a.pl, a.pr, a.tp);
  const int64_t ntot = a.off[a.nEnv];
  TO *out = (TO *)a.AAout;
  for (int64_t e = blockIdx.x; e < a.nEnv; e += gridDim.x) {
    const int64_t o0 = a.off[e], o1 = a.off[e + 1];
    if (o0 < 0 || o1 < o0 || o1 > ntot) {
      if (tid == 0) atomicOr(a.status, ACE_STATUS_BAD_OFFSETS);
      continue;
    }
    build_A<TE>(a, tb, o0, (int)(o1 - o0), a.chunkE, lay.slabE, s_an, s_aiy, s_amu, ssp, (TE *)(sm + lay.slab), AE);
    for (int64_t k = tid; k < a.nAA; k += nt) {
      const int ord = a.ord[k];
      cpx<TE> p = {Arith<TE>::one(), Arith<TE>::zero()};
      for (int t = 0; t < ord; ++t) p = cmul(p, AE[a.idx[(size_t)t * a.nAA + k]]);
      out[k * a.ldE + e] = (TO)lower<double>(p.re);
    }
    __syncthreads();
  }
}

// B[(e0 + e) * nB + b] = sum_k U[b, k] AA[k * ldE + e]  (genmul!, src/symmbasis.jl:248-264)
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

// Fused B = U real(AA) per environment, without AA in memory: phase 1 (A in
// shared memory), then each thread walks its entries (ace_sched.h
// build_urows): one AA function per entry, real(AA_k) = Re(prod A)
// (src/pibasis.jl:265-275) formed once and added with the entry's U values
// to the row accumulators of its group; a group's rows are written at its
// last entry (genmul!, src/symmbasis.jl:248-264).
template <typename TE>
__global__ void __launch_bounds__(128) ub_fused_kernel(EFArgs a, const uint4 *urec, const void *uval, int64_t ulen,
                                                       int64_t nB, double *B) {
  extern __shared__ __align__(16) unsigned char sm[];
  const EFLayout lay = ef_layout(a.ntab, a.nRs, a.L, a.nA, a.chunkE, 1, 0, 128, sizeof(TE), sizeof(TE), true);
  TE *tabE = (TE *)(sm + lay.tabE);
  int16_t *s_an = (int16_t *)(sm + lay.an);
  int16_t *s_aiy = (int16_t *)(sm + lay.aiy);
  int16_t *s_amu = (int16_t *)(sm + lay.amu);
  cpx<TE> *AE = (cpx<TE> *)(sm + lay.AE);
  int *ssp = (int *)(sm + lay.spc);
  const int tid = threadIdx.x, nt = blockDim.x;
  for (int i = tid; i < a.ntab; i += nt) tabE[i] = load_table<TE>(a.tabE, i);
  for (int i = tid; i < a.nA; i += nt) { s_an[i] = a.an[i]; s_aiy[i] = a.aiy[i]; s_amu[i] = a.amu[i]; }
  __syncthreads();
  Tables<TE> tb;
  tb.bind(tabE, a.nR, a.L, a.pl, a.pr, a.tp);
  const int64_t ntot = a.off[a.nEnv];
  const TE ze = Arith<TE>::zero();
  for (int64_t e = blockIdx.x; e < a.nEnv; e += gridDim.x) {
    const int64_t o0 = a.off[e], o1 = a.off[e + 1];
    if (o0 < 0 || o1 < o0 || o1 > ntot) {
      if (tid == 0) atomicOr(a.status, ACE_STATUS_BAD_OFFSETS);
      continue;
    }
    build_A<TE>(a, tb, o0, (int)(o1 - o0), a.chunkE, lay.slabE, s_an, s_aiy, s_amu, ssp, (TE *)(sm + lay.slab), AE);
    TE acc[UB_R];
#pragma unroll
    for (int i = 0; i < UB_R; ++i) acc[i] = ze;
    double *Be = B + e * nB;
    for (int64_t j = 0; j < ulen; ++j) {
      const int64_t slot = j * nt + tid;
      const uint4 rc = __ldg(urec + slot);
      if (!(rc.w >> 31)) break;  // padding only follows a thread's last entry
      const int ord = (rc.w >> 24) & 7;
      const uint32_t vw[3] = {rc.x, rc.y, rc.z};
      cpx<TE> p = {Arith<TE>::one(), ze};
#pragma unroll
      for (int t = 0; t < 6; ++t) {
        if (t < ord) {
          const cpx<TE> av = AE[(vw[t >> 1] >> (16 * (t & 1))) & 0xffff];
          p = (t == 0) ? av : cmul(p, av);
        }
      }
#pragma unroll
      for (int i = 0; i < UB_R; ++i) acc[i] = fmag(load_coef<TE>(uval, slot * UB_R + i), p.re, acc[i]);
      if ((rc.w >> 30) & 1u) {
        // write the group's r rows; the accumulators shift down so that only
        // r conversions to double (FP64-pipe work on GB300) are issued
        const int r = (int)((rc.w >> 27) & 7u) + 1;
        double *Bo = Be + (rc.w & ((1u << 24) - 1u));
        for (int i = 0; i < r; ++i) {
          Bo[i] = lower<double>(acc[0]);
#pragma unroll
          for (int q = 0; q < UB_R - 1; ++q) acc[q] = acc[q + 1];
          acc[UB_R - 1] = ze;
        }
#pragma unroll
        for (int i = 0; i < UB_R; ++i) acc[i] = ze;
      }
    }
    __syncthreads();
  }
}

// Kernel arguments for a context (host side).
inline EFArgs make_args(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr, const int32_t *sp,
                        double *E, double *G) {
  EFArgs a{};
  a.nEnv = nEnv; a.off = off; a.rr = rr; a.sp = sp; a.E = E; a.G = G;
  switch (ctx->prec) {
    case ACE_PREC_FP64: a.tabE = ctx->d_tabD; a.tabG = ctx->d_tabD; break;
    case ACE_PREC_FP32X2: a.tabE = ctx->d_tabDF; a.tabG = ctx->d_tabF; break;
    default: a.tabE = ctx->d_tabF; a.tabG = ctx->d_tabF; break;
  }
  a.ntab = ctx->ntab; a.nR = ctx->nR; a.L = ctx->L; a.pl = ctx->pl; a.pr = ctx->pr; a.tp = ctx->tp;
  a.nRs = ctx->learned ? ctx->mlpC : ctx->nR;
  a.Rext = ctx->learned ? ctx->d_Rext : nullptr;
  a.GR = nullptr;
  a.an = ctx->d_an; a.aiy = ctx->d_aiy; a.amu = ctx->d_amu;
  a.nA = ctx->nA; a.nspecies = ctx->nspecies;
  a.srec = ctx->d_srec; a.sc = ctx->d_sc; a.slen = ctx->slen;
  a.irec = ctx->d_irec; a.ic = ctx->d_ic; a.in = ctx->item_n;
  a.c0 = ctx->has_const ? ctx->ctilde[0] : 0.0;
  a.chunkE = ctx->chunkE; a.chunkG = ctx->chunkG; a.npriv = ctx->npriv;
  a.trec = ctx->d_trec; a.tc = ctx->d_tc;
  for (int w = 0; w < 5; ++w) a.twrow[w] = ctx->twrow[w];
  a.status = ctx->d_status;
  a.ord = ctx->d_ord; a.idx = ctx->d_idx; a.nAA = ctx->nAA;
  return a;
}

}  // namespace ace
