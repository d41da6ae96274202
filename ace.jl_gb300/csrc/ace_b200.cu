// ace_b200.cu -- libace_b200: C ABI, context management and host-side
// validation of the GB300 ACE evaluator.  Kernels live in ace_kernels.cuh.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <functional>
#include <string>
#include <vector>

#include "../../include/ace_b200.h"
#include "ace_ctx.h"
#include "ace_phi.cuh"
#include "ace_sched.h"

using namespace ace;

static thread_local std::string g_create_error;

#define ACE_CUDA(call)                                                            \
  do {                                                                            \
    cudaError_t _e = (call);                                                      \
    if (_e != cudaSuccess) {                                                      \
      return ctx_fail(ctx, ACE_ERR_CUDA, std::string(#call) + ": " + cudaGetErrorString(_e)); \
    }                                                                             \
  } while (0)

static int ctx_fail(ace_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg; else g_create_error = msg;
  return code;
}

template <typename T> static int upload(ace_ctx *ctx, T **dst, const T *src, size_t n) {
  *dst = nullptr;
  if (n == 0) return ACE_OK;
  ACE_CUDA(cudaMalloc((void **)dst, n * sizeof(T)));
  ctx->allocs.push_back(*dst);
  ACE_CUDA(cudaMemcpy(*dst, src, n * sizeof(T), cudaMemcpyHostToDevice));
  return ACE_OK;
}

static int pack_coefs(ace_ctx *ctx, void *dst, int64_t n, const std::function<double(int64_t)> &val);

// Coefficient table (layout documented in ace_phi.cuh).
static std::vector<double> coef_table(const ace_spec_bundle *s, int L) {
  const int szP = size_p(L);
  std::vector<double> t;
  t.insert(t.end(), s->rA, s->rA + s->nR);
  t.insert(t.end(), s->rB, s->rB + s->nR);
  t.insert(t.end(), s->rC, s->rC + s->nR);
  std::vector<double> A(szP, 0.0), B(szP, 0.0), C(L + 1, 0.0), D(L + 1, 0.0);
  if (L >= 1) { C[1] = std::sqrt(3.0); D[1] = -std::sqrt(1.5); }
  for (int l = 2; l <= L; ++l) {
    double ls = double(l * l), lm1s = double((l - 1) * (l - 1));
    for (int m = 0; m <= l - 2; ++m) {
      double ms = double(m * m);
      A[idx_p(l, m)] = std::sqrt((4 * ls - 1.0) / (ls - ms));
      B[idx_p(l, m)] = -std::sqrt((lm1s - ms) / (4 * lm1s - 1.0));
    }
    C[l] = std::sqrt(double(2 * (l - 1) + 3));
    D[l] = -std::sqrt(1.0 + 0.5 / l);
  }
  t.insert(t.end(), A.begin(), A.end());
  t.insert(t.end(), B.begin(), B.end());
  t.insert(t.end(), C.begin(), C.end());
  t.insert(t.end(), D.begin(), D.end());
  const double k[7] = {s->tl, s->tr, 1.0 + s->r0, std::sqrt(3.0), std::sqrt(1.5), std::sqrt(0.5 / M_PI),
                       1.0 / std::sqrt(2.0)};
  t.insert(t.end(), k, k + 7);
  return t;
}

static int validate_spec(const ace_spec_bundle *s, std::string &why) {
  if (!s) { why = "spec is NULL"; return ACE_ERR_INVALID; }
  if (s->version != ACE_SPEC_VERSION) { why = "spec version mismatch"; return ACE_ERR_INVALID; }
  if (s->nR < 1 || s->nR > ACE_MAX_NR) { why = "nR out of range [1, 32]"; return ACE_ERR_UNSUPPORTED; }
  if (!s->rA || !s->rB || !s->rC) { why = "radial coefficients missing"; return ACE_ERR_INVALID; }
  if (s->tp < 0 || s->tp > 8 || s->pl < 0 || s->pl > 8 || s->pr < 0 || s->pr > 8) {
    why = "transform/envelope powers out of range"; return ACE_ERR_UNSUPPORTED;
  }
  if (s->nA < 1 || s->nA > 65535) { why = "nA out of range [1, 65535]"; return ACE_ERR_UNSUPPORTED; }
  if (!s->a_n || !s->a_l || !s->a_m) { why = "A spec arrays missing"; return ACE_ERR_INVALID; }
  if (s->nspecies < 1 || s->nspecies > 255) { why = "nspecies out of range [1, 255]"; return ACE_ERR_UNSUPPORTED; }
  if (s->nspecies > 1 && !s->a_mu) { why = "a_mu required for more than one species"; return ACE_ERR_INVALID; }
  for (int i = 0; i < s->nA; ++i) {
    if (s->a_n[i] < 0 || s->a_n[i] >= s->nR) { why = "a_n out of range"; return ACE_ERR_INVALID; }
    if (s->a_l[i] < 0 || s->a_l[i] > ACE_MAX_L) { why = "a_l out of range [0, 20]"; return ACE_ERR_UNSUPPORTED; }
    if (s->a_m[i] < -s->a_l[i] || s->a_m[i] > s->a_l[i]) { why = "|a_m| > a_l"; return ACE_ERR_INVALID; }
    if (s->a_mu && (s->a_mu[i] < 0 || s->a_mu[i] >= s->nspecies)) { why = "a_mu out of range"; return ACE_ERR_INVALID; }
  }
  if (s->nAA < 1 || s->maxord < 1 || s->maxord > ACE_MAX_ORD) { why = "nAA/maxord out of range (maxord <= 6)"; return ACE_ERR_UNSUPPORTED; }
  if (!s->orders || !s->iAA2iA) { why = "AA spec arrays missing"; return ACE_ERR_INVALID; }
  for (int64_t k = 0; k < s->nAA; ++k) {
    int o = s->orders[k];
    if (o < 0 || o > s->maxord) { why = "orders out of range"; return ACE_ERR_INVALID; }
    if (o == 0 && k != 0) { why = "only the first AA function may have order 0"; return ACE_ERR_INVALID; }
    for (int t = 0; t < o; ++t) {
      int v = s->iAA2iA[k * s->maxord + t];
      if (v < 0 || v >= s->nA) { why = "iAA2iA entry out of range"; return ACE_ERR_INVALID; }
    }
  }
  if (s->nB < 0) { why = "nB < 0"; return ACE_ERR_INVALID; }
  if (s->nB > 0) {
    if (!s->U_indptr || !s->U_indices || !s->U_data) { why = "U arrays missing"; return ACE_ERR_INVALID; }
    if (s->U_indptr[0] != 0) { why = "U_indptr[0] != 0"; return ACE_ERR_INVALID; }
    for (int64_t b = 0; b < s->nB; ++b)
      if (s->U_indptr[b + 1] < s->U_indptr[b]) { why = "U_indptr not monotone"; return ACE_ERR_INVALID; }
    for (int64_t k = 0; k < s->U_indptr[s->nB]; ++k)
      if (s->U_indices[k] < 0 || s->U_indices[k] >= s->nAA) { why = "U index out of range"; return ACE_ERR_INVALID; }
  }
  return ACE_OK;
}

extern "C" int ace_ctx_create(const ace_spec_bundle *s, int32_t prec, int32_t device, ace_ctx **out) {
  if (!out) return ctx_fail(nullptr, ACE_ERR_INVALID, "out is NULL");
  *out = nullptr;
  std::string why;
  int rc = validate_spec(s, why);
  if (rc != ACE_OK) return ctx_fail(nullptr, rc, why);
  if (prec == ACE_PREC_FP32_BF16X3)
    return ctx_fail(nullptr, ACE_ERR_UNSUPPORTED,
                    "precision mode ACE_PREC_FP32_BF16X3 (split-BF16 tensor-core U*AA) is not built");
  if (prec != ACE_PREC_FP64 && prec != ACE_PREC_FP32 && prec != ACE_PREC_FP32X2 && prec != ACE_PREC_FP32_COMP)
    return ctx_fail(nullptr, ACE_ERR_UNSUPPORTED, "precision mode not supported");
  // the compensated form is the double-float form except for its
  // single-property energy/force kernel
  const bool comp = (prec == ACE_PREC_FP32_COMP);
  if (comp) prec = ACE_PREC_FP32X2;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev)
    return ctx_fail(nullptr, ACE_ERR_CUDA, "no such CUDA device");
  ace_ctx *ctx = new ace_ctx();
  ctx->device = device;
  ctx->prec = prec;
  ctx->comp = comp;
  ctx->guard_tol = comp ? 1e-6 : 0.0;
  ctx->nR = s->nR; ctx->nA = s->nA; ctx->nAA = s->nAA; ctx->nB = s->nB;
  ctx->maxord = s->maxord; ctx->nspecies = s->nspecies;
  ctx->pl = s->pl; ctx->pr = s->pr; ctx->tp = s->tp;
  ctx->tl = s->tl; ctx->tr = s->tr; ctx->r0 = s->r0;
  int L = 0;
  for (int i = 0; i < s->nA; ++i) L = std::max(L, s->a_l[i]);
  ctx->L = L;
  auto fail = [&](int code) { ace_ctx_destroy(ctx); return code; };
  if (cudaSetDevice(device) != cudaSuccess) { g_create_error = "cudaSetDevice failed"; return fail(ACE_ERR_CUDA); }
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) {
    g_create_error = "cudaGetDeviceProperties failed";
    return fail(ACE_ERR_CUDA);
  }
  ctx->nsm = prop.multiProcessorCount;
  ctx->smem_optin = (int)prop.sharedMemPerBlockOptin;

  // coefficient tables in double, float and double-float
  std::vector<double> tabD = coef_table(s, L);
  std::vector<float> tabF(tabD.begin(), tabD.end());
  std::vector<float> tabDF(2 * tabD.size());
  for (size_t i = 0; i < tabD.size(); ++i) {
    float h = (float)tabD[i];
    tabDF[2 * i] = h;
    tabDF[2 * i + 1] = (float)(tabD[i] - (double)h);
  }
  ctx->ntab = (int)tabD.size();
  // A spec
  std::vector<int16_t> an(s->nA), aiy(s->nA), amu(s->nA, 0);
  for (int i = 0; i < s->nA; ++i) {
    an[i] = (int16_t)s->a_n[i];
    aiy[i] = (int16_t)idx_y(s->a_l[i], s->a_m[i]);
    if (s->a_mu) amu[i] = (int16_t)s->a_mu[i];
  }
  // AA spec for the flat-product (basis) path: orders and SoA indices idx[t * nAA + k]
  std::vector<uint8_t> ord(s->nAA);
  std::vector<uint16_t> idx((size_t)s->maxord * s->nAA, 0);
  for (int64_t k = 0; k < s->nAA; ++k) {
    ord[k] = (uint8_t)s->orders[k];
    for (int t = 0; t < s->orders[k]; ++t) idx[(size_t)t * s->nAA + k] = (uint16_t)s->iAA2iA[k * s->maxord + t];
  }
  ctx->has_const = (s->orders[0] == 0);
  if ((rc = upload(ctx, &ctx->d_tabD, tabD.data(), tabD.size())) ||
      (rc = upload(ctx, &ctx->d_tabF, tabF.data(), tabF.size())) ||
      (rc = upload(ctx, &ctx->d_tabDF, tabDF.data(), tabDF.size())) ||
      (rc = upload(ctx, &ctx->d_an, an.data(), an.size())) ||
      (rc = upload(ctx, &ctx->d_aiy, aiy.data(), aiy.size())) ||
      (rc = upload(ctx, &ctx->d_amu, amu.data(), amu.size())) ||
      (rc = upload(ctx, &ctx->d_ord, ord.data(), ord.size())) ||
      (rc = upload(ctx, &ctx->d_idx, idx.data(), idx.size()))) {
    g_create_error = ctx->err;
    return fail(rc);
  }
  // correlation schedule
  {
    Schedule sch = build_schedule(s->nA, s->a_n, s->a_l, s->a_m, s->a_mu, s->nAA, s->maxord, s->orders,
                                  s->iAA2iA, s->nB, s->U_indptr, s->U_indices, s->U_data, ctx->nt);
    Interleaved il = interleave(sch, ctx->nt);
    ctx->sn = sch.n;
    ctx->halved = sch.halved;
    ctx->apartner = sch.partner;
    ctx->amsign = sch.msign;
    ctx->sched_nodes = sch.nodes;
    ctx->slen = il.len;
    const int64_t nslot = std::max<int64_t>(il.len * ctx->nt, 1);
    ctx->sslot.assign(nslot, -1);
    ctx->sw.assign(nslot, 0);
    for (int64_t j = 0; j < il.len * ctx->nt; ++j)
      if (il.perm[j] >= 0) { ctx->sslot[j] = sch.k[il.perm[j]]; ctx->sw[j] = sch.w[il.perm[j]]; }
    if (il.rec.empty()) il.rec.assign(8, 0);
    if ((rc = upload(ctx, (uint16_t **)&ctx->d_srec, il.rec.data(), il.rec.size()))) {
      g_create_error = ctx->err;
      return fail(rc);
    }
    const size_t csz = (prec == ACE_PREC_FP64) ? 8 : (prec == ACE_PREC_FP32X2 ? 8 : 4);
    // item schedule
    const char *kenv = getenv("ACE_B200_KERNEL");
    // (the compensated form exists on the item family of schedules only)
    ctx->use_items = comp || !(kenv && std::string(kenv) == "trie");
    ItemSchedule its = build_items(sch, ctx->nt);
    ctx->item_n = its.n;
    ctx->ik.assign((size_t)(ITEM_G + 1) * its.n, -1);
    ctx->iw.assign((size_t)(ITEM_G + 1) * its.n, 0);
    for (int64_t f = 0; f < its.n; ++f) {
      ctx->ik[f] = its.kown[f];
      ctx->iw[f] = its.wown[f];
      for (int g = 0; g < ITEM_G; ++g) {
        ctx->ik[(size_t)(g + 1) * its.n + f] = its.kleaf[(size_t)f * ITEM_G + g];
        ctx->iw[(size_t)(g + 1) * its.n + f] = its.wleaf[(size_t)f * ITEM_G + g];
      }
    }
    if ((rc = upload(ctx, (uint16_t **)&ctx->d_irec, its.rec.data(), its.rec.size()))) {
      g_create_error = ctx->err;
      return fail(rc);
    }
    if (cudaMalloc(&ctx->d_ic, ctx->ik.size() * csz) != cudaSuccess) {
      g_create_error = "cudaMalloc failed";
      return fail(ACE_ERR_ALLOC);
    }
    ctx->allocs.push_back(ctx->d_ic);
    if (cudaMemset(ctx->d_ic, 0, ctx->ik.size() * csz) != cudaSuccess) {
      g_create_error = "cudaMemset failed";
      return fail(ACE_ERR_CUDA);
    }
    // task schedule (orders >= 3)
    if (s->maxord >= 3 && ctx->nt == 128) {
      TaskSchedule ts = build_tasks(sch, ctx->nt / 32);
      ctx->has_tasks = ctx->use_tasks = ts.rows > 0;
      ctx->trows = ts.rows;
      for (int w = 0; w <= ts.nwarps && w < 5; ++w) ctx->twrow[w] = ts.wrow[w];
      ctx->tk = std::move(ts.ck);
      ctx->tw = std::move(ts.cw);
      if (ctx->has_tasks) {
        if ((rc = upload(ctx, (uint16_t **)&ctx->d_trec, ts.rec.data(), ts.rec.size()))) {
          g_create_error = ctx->err;
          return fail(rc);
        }
        // coefficients in the energy type (a compensated context: also in
        // FP32 for its own kernels; the double-float ones serve its
        // re-evaluations)
        for (int copy = 0; copy < (comp ? 2 : 1); ++copy) {
          const size_t tsz = copy ? 4 : csz;
          void **dst = copy ? (void **)&ctx->d_tc32 : &ctx->d_tc;
          if (cudaMalloc(dst, ctx->tk.size() * tsz) != cudaSuccess) {
            g_create_error = "cudaMalloc failed";
            return fail(ACE_ERR_ALLOC);
          }
          ctx->allocs.push_back(*dst);
          if (cudaMemset(*dst, 0, ctx->tk.size() * tsz) != cudaSuccess) {
            g_create_error = "cudaMemset failed";
            return fail(ACE_ERR_CUDA);
          }
        }
      }
      if (const char *kenv2 = getenv("ACE_B200_KERNEL"))
        if (std::string(kenv2) == "items" || std::string(kenv2) == "trie") ctx->use_tasks = false;
    }
    if (comp) {
      if (cudaMalloc((void **)&ctx->d_ic32, ctx->ik.size() * sizeof(float)) != cudaSuccess) {
        g_create_error = "cudaMalloc failed";
        return fail(ACE_ERR_ALLOC);
      }
      ctx->allocs.push_back(ctx->d_ic32);
      if (cudaMemset(ctx->d_ic32, 0, ctx->ik.size() * sizeof(float)) != cudaSuccess) {
        g_create_error = "cudaMemset failed";
        return fail(ACE_ERR_CUDA);
      }
    }
    if (cudaMalloc(&ctx->d_sc, nslot * csz) != cudaSuccess) {
      g_create_error = "cudaMalloc failed";
      return fail(ACE_ERR_ALLOC);
    }
    ctx->allocs.push_back(ctx->d_sc);
    if (cudaMemset(ctx->d_sc, 0, nslot * csz) != cudaSuccess) {
      g_create_error = "cudaMemset failed";
      return fail(ACE_ERR_CUDA);
    }
  }
  // U (host copy for c~ = U^T c; device copy for the basis path)
  if (s->nB > 0) {
    int64_t nnz = s->U_indptr[s->nB];
    ctx->U_indptr.assign(s->U_indptr, s->U_indptr + s->nB + 1);
    ctx->U_indices.assign(s->U_indices, s->U_indices + nnz);
    ctx->U_data.assign(s->U_data, s->U_data + nnz);
    std::vector<float> uf(ctx->U_data.begin(), ctx->U_data.end());
    if ((rc = upload(ctx, &ctx->d_Uptr, s->U_indptr, s->nB + 1)) ||
        (rc = upload(ctx, &ctx->d_Uidx, s->U_indices, nnz)) ||
        (rc = upload(ctx, &ctx->d_UvalD, s->U_data, nnz)) ||
        (rc = upload(ctx, &ctx->d_UvalF, uf.data(), uf.size()))) {
      g_create_error = ctx->err;
      return fail(rc);
    }
    // fused basis table (measured faster than the AA-scratch path in every
    // form); ACE_B200_BASIS=materialised keeps the AA-scratch path
    const char *benv = getenv("ACE_B200_BASIS");
    ctx->fused_basis = true;
    if (benv && std::string(benv) == "materialised") ctx->fused_basis = false;
    if (benv && std::string(benv) == "fused") ctx->fused_basis = true;
    if (s->nB >= (int64_t(1) << 24)) ctx->fused_basis = false;
    if (ctx->fused_basis) {
      URows ur = build_urows(s->nB, s->U_indptr, s->U_indices, s->U_data, s->orders, s->iAA2iA, s->maxord, 128,
                             ctx->apartner);
      ctx->ulen = ur.len;
      const size_t csz = (prec == ACE_PREC_FP32 || prec == ACE_PREC_FP32_BF16X3) ? 4 : 8;
      if ((rc = upload(ctx, (uint32_t **)&ctx->d_urec, ur.rec.data(), ur.rec.size()))) {
        g_create_error = ctx->err;
        return fail(rc);
      }
      if (cudaMalloc(&ctx->d_uval, std::max<size_t>(ur.val.size(), 1) * csz) != cudaSuccess) {
        g_create_error = "cudaMalloc failed";
        return fail(ACE_ERR_ALLOC);
      }
      ctx->allocs.push_back(ctx->d_uval);
      rc = pack_coefs(ctx, ctx->d_uval, (int64_t)ur.val.size(), [&](int64_t j) { return ur.val[j]; });
      if (rc != ACE_OK) {
        g_create_error = ctx->err;
        return fail(rc);
      }
    }
  }
  // status word
  if (cudaMalloc((void **)&ctx->d_status, sizeof(int)) != cudaSuccess) {
    g_create_error = "cudaMalloc failed";
    return fail(ACE_ERR_ALLOC);
  }
  ctx->allocs.push_back(ctx->d_status);
  if (cudaMemset(ctx->d_status, 0, sizeof(int)) != cudaSuccess) {
    g_create_error = "cudaMemset failed";
    return fail(ACE_ERR_CUDA);
  }
  ctx->ctilde.assign(s->nAA, 0.0);
  if (cudaMallocHost((void **)&ctx->h_status, sizeof(int)) != cudaSuccess) {
    g_create_error = "cudaMallocHost failed";
    return fail(ACE_ERR_ALLOC);
  }
  if (cudaDeviceSynchronize() != cudaSuccess) { g_create_error = "device sync failed"; return fail(ACE_ERR_CUDA); }
  // a fixed shared region (KB) instead of the default, as ace_autotune would
  // choose it (for profiling one configuration)
  if (const char *renv = getenv("ACE_B200_REGION_KB")) ctx->region_kb = std::max(8, std::min(96, atoi(renv)));
  rc = kernels_prepare(ctx);
  if (rc != ACE_OK) { g_create_error = ctx->err; return fail(rc); }
  // the allocation-free basis entry point's scratch address (its outcome is
  // reported by ace_basis_noalloc, not here)
  noalloc_prepare(ctx);
  *out = ctx;
  return ACE_OK;
}

extern "C" int ace_ctx_destroy(ace_ctx *ctx) {
  if (!ctx) return ACE_OK;
  cudaSetDevice(ctx->device);
  cudaDeviceSynchronize();
  for (void *p : ctx->allocs) cudaFree(p);
  if (ctx->d_stage) cudaFree(ctx->d_stage);
  if (ctx->d_scratch) cudaFree(ctx->d_scratch);
  if (ctx->d_gest) cudaFree(ctx->d_gest);
  if (ctx->d_glist) cudaFree(ctx->d_glist);
  if (ctx->d_wstage) cudaFree(ctx->d_wstage);
  if (ctx->d_ic_multi) cudaFree(ctx->d_ic_multi);
  for (cudaStream_t st : {ctx->s_in, ctx->s_comp, ctx->s_out})
    if (st) cudaStreamDestroy(st);
  for (cudaEvent_t ev : ctx->pipe_ev) cudaEventDestroy(ev);
  if (ctx->d_mlp) cudaFree(ctx->d_mlp);
  if (ctx->d_Rext) cudaFree(ctx->d_Rext);
  if (ctx->h_status) cudaFreeHost(ctx->h_status);
  delete ctx;
  return ACE_OK;
}

// Pack w * c~ in schedule order, in the energy type of the precision mode.
static int pack_coefs(ace_ctx *ctx, void *dst, int64_t n, const std::function<double(int64_t)> &val) {
  if (ctx->prec == ACE_PREC_FP64) {
    std::vector<double> c(n);
    for (int64_t j = 0; j < n; ++j) c[j] = val(j);
    ACE_CUDA(cudaMemcpy(dst, c.data(), n * 8, cudaMemcpyHostToDevice));
  } else if (ctx->prec == ACE_PREC_FP32X2) {
    std::vector<float> c(2 * n);
    for (int64_t j = 0; j < n; ++j) {
      const double v = val(j);
      const float h = (float)v;
      c[2 * j] = h;
      c[2 * j + 1] = (float)(v - (double)h);
    }
    ACE_CUDA(cudaMemcpy(dst, c.data(), n * 8, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> c(n);
    for (int64_t j = 0; j < n; ++j) c[j] = (float)val(j);
    ACE_CUDA(cudaMemcpy(dst, c.data(), n * 4, cudaMemcpyHostToDevice));
  }
  return ACE_OK;
}

static int push_ctilde(ace_ctx *ctx) {
  ACE_CUDA(cudaSetDevice(ctx->device));
  int rc = pack_coefs(ctx, ctx->d_ic, (int64_t)ctx->ik.size(), [&](int64_t j) {
    return ctx->ik[j] < 0 ? 0.0 : ctx->iw[j] * ctx->ctilde[ctx->ik[j]];
  });
  if (rc) return rc;
  if (ctx->comp) {
    std::vector<float> c(ctx->ik.size());
    for (size_t j = 0; j < c.size(); ++j) c[j] = ctx->ik[j] < 0 ? 0.f : (float)(ctx->iw[j] * ctx->ctilde[ctx->ik[j]]);
    ACE_CUDA(cudaMemcpy(ctx->d_ic32, c.data(), c.size() * sizeof(float), cudaMemcpyHostToDevice));
  }
  if (ctx->has_tasks) {
    auto tval = [&](int64_t j) { return ctx->tk[j] < 0 ? 0.0 : ctx->tw[j] * ctx->ctilde[ctx->tk[j]]; };
    if (ctx->comp) {
      std::vector<float> c(ctx->tk.size());
      for (size_t j = 0; j < c.size(); ++j) c[j] = (float)tval((int64_t)j);
      ACE_CUDA(cudaMemcpy(ctx->d_tc32, c.data(), c.size() * sizeof(float), cudaMemcpyHostToDevice));
    }
    rc = pack_coefs(ctx, ctx->d_tc, (int64_t)ctx->tk.size(), tval);
    if (rc) return rc;
  }
  const int64_t n = (int64_t)ctx->sslot.size();
  auto val = [&](int64_t j) { return ctx->sslot[j] < 0 ? 0.0 : ctx->sw[j] * ctx->ctilde[ctx->sslot[j]]; };
  if (ctx->prec == ACE_PREC_FP64) {
    std::vector<double> c(n);
    for (int64_t j = 0; j < n; ++j) c[j] = val(j);
    ACE_CUDA(cudaMemcpy(ctx->d_sc, c.data(), n * 8, cudaMemcpyHostToDevice));
  } else if (ctx->prec == ACE_PREC_FP32X2) {
    std::vector<float> c(2 * n);
    for (int64_t j = 0; j < n; ++j) {
      const double v = val(j);
      const float h = (float)v;
      c[2 * j] = h;
      c[2 * j + 1] = (float)(v - (double)h);
    }
    ACE_CUDA(cudaMemcpy(ctx->d_sc, c.data(), n * 8, cudaMemcpyHostToDevice));
  } else {
    std::vector<float> c(n);
    for (int64_t j = 0; j < n; ++j) c[j] = (float)val(j);
    ACE_CUDA(cudaMemcpy(ctx->d_sc, c.data(), n * 4, cudaMemcpyHostToDevice));
  }
  return ACE_OK;
}

extern "C" int ace_set_params(ace_ctx *ctx, const double *c, int64_t nB) {
  if (!ctx || !c) return ctx_fail(ctx, ACE_ERR_INVALID, "NULL argument");
  if (nB != ctx->nB) return ctx_fail(ctx, ACE_ERR_INVALID, "length of c != nB");
  // c~ = U^T c (genmul! with the transposed U, src/evaluator.jl:59-60)
  std::fill(ctx->ctilde.begin(), ctx->ctilde.end(), 0.0);
  for (int64_t b = 0; b < nB; ++b)
    for (int64_t k = ctx->U_indptr[b]; k < ctx->U_indptr[b + 1]; ++k)
      ctx->ctilde[ctx->U_indices[k]] += ctx->U_data[k] * c[b];
  return push_ctilde(ctx);
}

extern "C" int ace_set_params_multi(ace_ctx *ctx, const double *c, int64_t nB, int32_t nprop) {
  if (!ctx || !c) return ctx_fail(ctx, ACE_ERR_INVALID, "NULL argument");
  if (nB != ctx->nB) return ctx_fail(ctx, ACE_ERR_INVALID, "length of c != nB");
  if (nprop < 1 || nprop > 4096) return ctx_fail(ctx, ACE_ERR_INVALID, "nprop out of range [1, 4096]");
  if (!ctx->use_items) return ctx_fail(ctx, ACE_ERR_UNSUPPORTED, "multi-property models need the item schedule");
  ACE_CUDA(cudaSetDevice(ctx->device));
  ctx->cplx = false;
  ctx->ctilde_multi.assign((size_t)nprop * ctx->nAA, 0.0);
  for (int p = 0; p < nprop; ++p) {
    double *ct = ctx->ctilde_multi.data() + (size_t)p * ctx->nAA;
    const double *cp = c + (size_t)p * nB;
    for (int64_t b = 0; b < nB; ++b)
      for (int64_t k = ctx->U_indptr[b]; k < ctx->U_indptr[b + 1]; ++k) ct[ctx->U_indices[k]] += ctx->U_data[k] * cp[b];
  }
  const size_t csz = (ctx->prec == ACE_PREC_FP64 || ctx->prec == ACE_PREC_FP32X2) ? 8 : 4;
  const size_t per = ctx->ik.size() * csz;
  if (ctx->d_ic_multi && nprop > ctx->nprop) {
    cudaFree(ctx->d_ic_multi);
    ctx->d_ic_multi = nullptr;
  }
  if (!ctx->d_ic_multi && cudaMalloc(&ctx->d_ic_multi, per * nprop) != cudaSuccess)
    return ctx_fail(ctx, ACE_ERR_ALLOC, "coefficient allocation failed");
  ctx->nprop = nprop;
  for (int p = 0; p < nprop; ++p) {
    const double *ct = ctx->ctilde_multi.data() + (size_t)p * ctx->nAA;
    int rc = pack_coefs(ctx, (char *)ctx->d_ic_multi + p * per, (int64_t)ctx->ik.size(), [&](int64_t j) {
      return ctx->ik[j] < 0 ? 0.0 : ctx->iw[j] * ct[ctx->ik[j]];
    });
    if (rc) return rc;
  }
  return ACE_OK;
}

extern "C" int ace_set_ctilde_complex(ace_ctx *ctx, const double *ct, int64_t nAA, int32_t nprop) {
  if (!ctx || !ct) return ctx_fail(ctx, ACE_ERR_INVALID, "NULL argument");
  if (nAA != ctx->nAA) return ctx_fail(ctx, ACE_ERR_INVALID, "length of ctilde != nAA");
  if (nprop < 1 || nprop > 4096) return ctx_fail(ctx, ACE_ERR_INVALID, "nprop out of range [1, 4096]");
  ACE_CUDA(cudaSetDevice(ctx->device));
  const size_t csz = (ctx->prec == ACE_PREC_FP64 || ctx->prec == ACE_PREC_FP32X2) ? 8 : 4;
  const int64_t ns = (int64_t)ctx->ik.size();
  const size_t per = 2 * (size_t)ns * csz;
  if (ctx->d_ic_multi && (nprop > ctx->nprop || !ctx->cplx)) {
    cudaFree(ctx->d_ic_multi);
    ctx->d_ic_multi = nullptr;
  }
  if (!ctx->d_ic_multi && cudaMalloc(&ctx->d_ic_multi, per * nprop) != cudaSuccess)
    return ctx_fail(ctx, ACE_ERR_ALLOC, "coefficient allocation failed");
  ctx->cplx = true;
  ctx->nprop = nprop;
  ctx->ctilde_multi.assign((size_t)nprop * ctx->nAA, 0.0);
  for (int p = 0; p < nprop; ++p) {
    const double *cp = ct + (size_t)p * 2 * nAA;
    for (int64_t k = 0; k < nAA; ++k) ctx->ctilde_multi[(size_t)p * nAA + k] = cp[2 * k];
    // a slot of weight 2 stands for k and its m-reversed partner k':
    // Re(c_k AA_k + c_k' AA_k') = Re((c_k + s_k conj(c_k')) AA_k)
    auto coef = [&](int64_t j, bool im) {
      const int64_t k = ctx->ik[j];
      if (k < 0) return 0.0;
      double re = cp[2 * k], ii = cp[2 * k + 1];
      if (ctx->iw[j] == 2) {
        const int64_t q = ctx->apartner[k];
        re += ctx->amsign[k] * cp[2 * q];
        ii -= ctx->amsign[k] * cp[2 * q + 1];
      }
      return im ? ii : re;
    };
    int rc = pack_coefs(ctx, (char *)ctx->d_ic_multi + p * per, 2 * ns,
                        [&](int64_t j) { return j < ns ? coef(j, false) : coef(j - ns, true); });
    if (rc) return rc;
  }
  return ACE_OK;
}

extern "C" int ace_set_ctilde(ace_ctx *ctx, const double *ct, int64_t nAA) {
  if (!ctx || !ct) return ctx_fail(ctx, ACE_ERR_INVALID, "NULL argument");
  if (nAA != ctx->nAA) return ctx_fail(ctx, ACE_ERR_INVALID, "length of ctilde != nAA");
  ctx->ctilde.assign(ct, ct + nAA);
  return push_ctilde(ctx);
}

// Host-side validation of host inputs (the library never reads outside the
// CSR extent it is given; device inputs are checked inside the kernels).
// species an input batch carries: the spec's, or the radial MLP's in the
// learned form (whose spec is single-species)
static int input_species(const ace_ctx *ctx) { return ctx->learned ? ctx->mlpS : ctx->nspecies; }

static int validate_offsets(ace_ctx *ctx, int64_t nEnv, const int64_t *off) {
  if (nEnv < 0) return ctx_fail(ctx, ACE_ERR_INVALID, "nEnv < 0");
  if (off[0] != 0) return ctx_fail(ctx, ACE_ERR_INVALID, "offsets[0] != 0");
  for (int64_t e = 0; e < nEnv; ++e)
    if (off[e + 1] < off[e]) return ctx_fail(ctx, ACE_ERR_INVALID, "offsets not monotone");
  return ACE_OK;
}

// positions and species of neighbours [j0, j1)
static int validate_range(ace_ctx *ctx, int64_t j0, int64_t j1, const double *rr, const int32_t *sp) {
  for (int64_t j = j0; j < j1; ++j) {
    double x = rr[3 * j], y = rr[3 * j + 1], z = rr[3 * j + 2];
    if (!std::isfinite(x) || !std::isfinite(y) || !std::isfinite(z))
      return ctx_fail(ctx, ACE_ERR_INVALID, "non-finite position");
    if (x == 0.0 && y == 0.0 && z == 0.0)
      return ctx_fail(ctx, ACE_ERR_INVALID, "neighbour at the centre (r == 0)");
  }
  const int nsp = input_species(ctx);
  if (nsp > 1) {
    if (!sp) return ctx_fail(ctx, ACE_ERR_INVALID, "species required for a multi-species spec");
    for (int64_t j = j0; j < j1; ++j)
      if (sp[j] < 0 || sp[j] >= nsp) return ctx_fail(ctx, ACE_ERR_INVALID, "species out of range");
  }
  return ACE_OK;
}

static int validate_inputs(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr,
                           const int32_t *sp) {
  int rc = validate_offsets(ctx, nEnv, off);
  if (rc) return rc;
  return validate_range(ctx, 0, off[nEnv], rr, sp);
}

static int ensure_stage(ace_ctx *ctx, size_t bytes) {
  if (bytes <= ctx->stage_bytes) return ACE_OK;
  if (ctx->d_stage) { cudaFree(ctx->d_stage); ctx->d_stage = nullptr; ctx->stage_bytes = 0; }
  size_t want = std::max(bytes, (size_t)(ctx->stage_bytes * 3 / 2));
  if (cudaMalloc(&ctx->d_stage, want) != cudaSuccess) return ctx_fail(ctx, ACE_ERR_ALLOC, "staging allocation failed");
  ctx->stage_bytes = want;
  return ACE_OK;
}

static size_t al256(size_t x) { return (x + 255) & ~size_t(255); }

static int read_status(ace_ctx *ctx, cudaStream_t st) {
  ACE_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->d_status, sizeof(int), cudaMemcpyDeviceToHost, st));
  ACE_CUDA(cudaStreamSynchronize(st));
  int s = *ctx->h_status;
  if (s != 0) {
    std::string m = "kernel status:";
    if (s & ACE_STATUS_BAD_OFFSETS) m += " bad offsets;";
    if (s & ACE_STATUS_BAD_SPECIES) m += " species out of range;";
    if (s & ACE_STATUS_BAD_POSITION) m += " bad position;";
    if (s & ACE_STATUS_SCRATCH) m += " scratch too small;";
    if (s & ACE_STATUS_TIMEOUT) m += " tensor-core wait timed out;";
    ctx->err = m;
    cudaMemsetAsync(ctx->d_status, 0, sizeof(int), st);
    cudaStreamSynchronize(st);
    return ACE_ERR_KERNEL;
  }
  return ACE_OK;
}

// Shared driver of the evaluation calls: stages host buffers when needed,
// launches `run`, copies outputs back.
template <typename Run>
static int drive(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                 const int32_t *species, int32_t flags, void *stream,
                 std::vector<std::pair<void *, size_t>> outs_host_bytes, Run run) {
  if (!ctx) return ACE_ERR_INVALID;
  if (nEnv < 0 || !offsets || !rr) return ctx_fail(ctx, ACE_ERR_INVALID, "NULL or negative argument");
  ACE_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = (cudaStream_t)stream;
  const bool din = flags & ACE_INPUTS_ON_DEVICE;
  const bool dout = flags & ACE_OUTPUTS_ON_DEVICE;
  const int64_t *d_off = offsets;
  const double *d_rr = rr;
  const int32_t *d_sp = species;
  int64_t nNbr = -1;
  if (!din) {
    int rc = validate_inputs(ctx, nEnv, offsets, rr, species);
    if (rc) return rc;
    nNbr = offsets[nEnv];
  } else if (input_species(ctx) > 1 && !species) {
    return ctx_fail(ctx, ACE_ERR_INVALID, "species required for a multi-species spec");
  }
  const int nsp = input_species(ctx);
  // staging: inputs (if host) + outputs (if host)
  size_t need = 0;
  size_t o_off = 0, o_rr = 0, o_sp = 0;
  if (!din) {
    o_off = need; need += al256((nEnv + 1) * sizeof(int64_t));
    o_rr = need; need += al256(std::max<int64_t>(nNbr, 1) * 3 * sizeof(double));
    if (species && nsp > 1) { o_sp = need; need += al256(std::max<int64_t>(nNbr, 1) * sizeof(int32_t)); }
  }
  std::vector<size_t> o_out(outs_host_bytes.size());
  if (!dout)
    for (size_t i = 0; i < outs_host_bytes.size(); ++i) { o_out[i] = need; need += al256(outs_host_bytes[i].second); }
  int rc = ensure_stage(ctx, need);
  if (rc) return rc;
  char *base = (char *)ctx->d_stage;
  // on a failure after work was issued the stream is drained before
  // returning, so no copy touches the caller's buffers after the call
  auto fail_drained = [&](int code, const std::string &msg) {
    cudaStreamSynchronize(st);
    return ctx_fail(ctx, code, msg);
  };
  if (!din) {
    cudaError_t ce = cudaMemcpyAsync(base + o_off, offsets, (nEnv + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, st);
    if (ce == cudaSuccess) ce = cudaMemcpyAsync(base + o_rr, rr, nNbr * 3 * sizeof(double), cudaMemcpyHostToDevice, st);
    d_off = (const int64_t *)(base + o_off);
    d_rr = (const double *)(base + o_rr);
    if (species && nsp > 1) {
      if (ce == cudaSuccess) ce = cudaMemcpyAsync(base + o_sp, species, nNbr * sizeof(int32_t), cudaMemcpyHostToDevice, st);
      d_sp = (const int32_t *)(base + o_sp);
    } else {
      d_sp = nullptr;
    }
    if (ce != cudaSuccess) return fail_drained(ACE_ERR_CUDA, std::string("input copy: ") + cudaGetErrorString(ce));
  } else if (nsp == 1) {
    d_sp = nullptr;
  }
  std::vector<void *> d_outs(outs_host_bytes.size());
  for (size_t i = 0; i < outs_host_bytes.size(); ++i)
    d_outs[i] = (dout || !outs_host_bytes[i].first) ? outs_host_bytes[i].first : (void *)(base + o_out[i]);
  rc = run(d_off, d_rr, d_sp, d_outs, st);
  if (rc) {
    if (!din) cudaStreamSynchronize(st);
    return rc;
  }
  if (!dout) {
    cudaError_t ce = cudaSuccess;
    for (size_t i = 0; i < outs_host_bytes.size() && ce == cudaSuccess; ++i)
      if (outs_host_bytes[i].first)
        ce = cudaMemcpyAsync(outs_host_bytes[i].first, d_outs[i], outs_host_bytes[i].second, cudaMemcpyDeviceToHost, st);
    if (ce != cudaSuccess) return fail_drained(ACE_ERR_CUDA, std::string("output copy: ") + cudaGetErrorString(ce));
  }
  if (!(flags & ACE_ASYNC) || !din || !dout) return read_status(ctx, st);
  return ACE_OK;
}

// Host buffers in and out, large batches: the batch is cut into chunks of
// environments (up to 8; ACE_B200_PIPE_CHUNKS overrides); chunk k+1 is
// validated on the host while chunk k's positions
// are copied in (copy stream), evaluated (compute stream) and its energies and
// gradients copied out (a second copy stream), so copies, host checks and
// kernels overlap.  An invalid chunk stops the pipeline; earlier chunks may
// then have been evaluated and their outputs written.
static constexpr int64_t PIPE_MIN_CHUNK = 4096;

static int ensure_pipeline(ace_ctx *ctx, int nchunk) {
  for (cudaStream_t *p : {&ctx->s_in, &ctx->s_comp, &ctx->s_out})
    if (!*p) ACE_CUDA(cudaStreamCreateWithFlags(p, cudaStreamNonBlocking));
  while ((int)ctx->pipe_ev.size() < 2 * nchunk) {
    cudaEvent_t ev;
    ACE_CUDA(cudaEventCreateWithFlags(&ev, cudaEventDisableTiming));
    ctx->pipe_ev.push_back(ev);
  }
  return ACE_OK;
}

static int energy_forces_pipelined(ace_ctx *ctx, int64_t nEnv, const int64_t *off, const double *rr,
                                   const int32_t *sp, double *E, double *G) {
  int rc = validate_offsets(ctx, nEnv, off);
  if (rc) return rc;
  const int64_t nNbr = off[nEnv];
  const int nsp = input_species(ctx);
  if (nsp > 1 && !sp) return ctx_fail(ctx, ACE_ERR_INVALID, "species required for a multi-species spec");
  const bool wsp = sp && nsp > 1;
  int maxchunk = 8;  // measured on GB300 (ord4/deg12, 100k envs): 4 / 8 / 16 / 32 chunks -> 2.74 / 2.82 / 2.74 / 2.68 M env/s
  if (const char *pc = getenv("ACE_B200_PIPE_CHUNKS")) maxchunk = std::max(2, std::min(64, atoi(pc)));
  const int nchunk = (int)std::max<int64_t>(2, std::min<int64_t>(maxchunk, nEnv / PIPE_MIN_CHUNK));
  ACE_CUDA(cudaSetDevice(ctx->device));
  if ((rc = ensure_pipeline(ctx, nchunk))) return rc;
  size_t need = 0;
  const size_t o_off = need; need += al256((nEnv + 1) * sizeof(int64_t));
  const size_t o_rr = need; need += al256(std::max<int64_t>(nNbr, 1) * 3 * sizeof(double));
  const size_t o_sp = need; if (wsp) need += al256(std::max<int64_t>(nNbr, 1) * sizeof(int32_t));
  const size_t o_E = need; need += al256(nEnv * sizeof(double));
  const size_t o_G = need; if (G) need += al256(std::max<int64_t>(nNbr, 1) * 3 * sizeof(double));
  if ((rc = ensure_stage(ctx, need))) return rc;
  // the compensated form's error estimates of every chunk (at offset e0)
  if (ctx->comp && (rc = guard_prepare(ctx, nEnv))) return rc;
  char *base = (char *)ctx->d_stage;
  int64_t *d_off = (int64_t *)(base + o_off);
  double *d_rr = (double *)(base + o_rr);
  int32_t *d_sp = wsp ? (int32_t *)(base + o_sp) : nullptr;
  double *d_E = (double *)(base + o_E);
  double *d_G = G ? (double *)(base + o_G) : nullptr;
  // a failure inside the loop stops issuing work; every stream is drained
  // before returning, so no copy into the caller's buffers outlives the call
  int err = ACE_OK;
  auto ck = [&](cudaError_t e, const char *what) {
    if (e != cudaSuccess && err == ACE_OK) err = ctx_fail(ctx, ACE_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
    return err == ACE_OK;
  };
  ck(cudaMemcpyAsync(d_off, off, (nEnv + 1) * sizeof(int64_t), cudaMemcpyHostToDevice, ctx->s_in), "offsets copy");
  for (int k = 0; k < nchunk && err == ACE_OK; ++k) {
    const int64_t e0 = nEnv * k / nchunk, e1 = nEnv * (k + 1) / nchunk;
    const int64_t j0 = off[e0], j1 = off[e1];
    if ((err = validate_range(ctx, j0, j1, rr, sp))) break;
    cudaEvent_t ev_in = ctx->pipe_ev[2 * k], ev_comp = ctx->pipe_ev[2 * k + 1];
    if (j1 > j0) {
      if (!ck(cudaMemcpyAsync(d_rr + 3 * j0, rr + 3 * j0, (j1 - j0) * 3 * sizeof(double), cudaMemcpyHostToDevice,
                              ctx->s_in), "positions copy"))
        break;
      if (wsp && !ck(cudaMemcpyAsync(d_sp + j0, sp + j0, (j1 - j0) * sizeof(int32_t), cudaMemcpyHostToDevice,
                                     ctx->s_in), "species copy"))
        break;
    }
    if (!ck(cudaEventRecord(ev_in, ctx->s_in), "event record") ||
        !ck(cudaStreamWaitEvent(ctx->s_comp, ev_in, 0), "stream wait"))
      break;
    ctx->guard_off = e0;
    err = launch_energy_forces(ctx, e1 - e0, d_off + e0, d_rr, d_sp, d_E + e0, d_G, ctx->s_comp);
    ctx->guard_off = 0;
    if (err) break;
    if (!ck(cudaEventRecord(ev_comp, ctx->s_comp), "event record") ||
        !ck(cudaStreamWaitEvent(ctx->s_out, ev_comp, 0), "stream wait"))
      break;
    if (!ck(cudaMemcpyAsync(E + e0, d_E + e0, (e1 - e0) * sizeof(double), cudaMemcpyDeviceToHost, ctx->s_out),
            "energies copy"))
      break;
    if (G && j1 > j0 &&
        !ck(cudaMemcpyAsync(G + 3 * j0, d_G + 3 * j0, (j1 - j0) * 3 * sizeof(double), cudaMemcpyDeviceToHost,
                            ctx->s_out), "gradients copy"))
      break;
  }
  const cudaError_t q_out = cudaStreamSynchronize(ctx->s_out);
  const cudaError_t q_comp = cudaStreamSynchronize(ctx->s_comp);
  const cudaError_t q_in = cudaStreamSynchronize(ctx->s_in);
  ck(q_out, "stream synchronize");
  ck(q_comp, "stream synchronize");
  ck(q_in, "stream synchronize");
  if (err) return err;
  return read_status(ctx, ctx->s_comp);
}

extern "C" int ace_energy_forces(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                                 const int32_t *species, double *E, double *dEdrr, int32_t flags,
                                 void *stream) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!E) return ctx_fail(ctx, ACE_ERR_INVALID, "E is NULL");
  if (!(flags & (ACE_INPUTS_ON_DEVICE | ACE_OUTPUTS_ON_DEVICE)) && !ctx->learned && offsets && rr &&
      nEnv >= 2 * PIPE_MIN_CHUNK)
    return energy_forces_pipelined(ctx, nEnv, offsets, rr, species, E, dEdrr);
  int64_t nNbr = (flags & ACE_INPUTS_ON_DEVICE) ? 0 : (offsets ? offsets[nEnv] : 0);
  if ((flags & ACE_INPUTS_ON_DEVICE) && dEdrr && !(flags & ACE_OUTPUTS_ON_DEVICE))
    return ctx_fail(ctx, ACE_ERR_INVALID, "host gradient output needs host inputs (the size is unknown)");
  std::vector<std::pair<void *, size_t>> outs = {{E, nEnv * sizeof(double)},
                                                 {dEdrr, (size_t)nNbr * 3 * sizeof(double)}};
  return drive(ctx, nEnv, offsets, rr, species, flags, stream, outs,
               [&](const int64_t *o, const double *x, const int32_t *s, std::vector<void *> &d, cudaStream_t st) {
                 return launch_energy_forces(ctx, nEnv, o, x, s, (double *)d[0], (double *)d[1], st);
               });
}

extern "C" int ace_energy_forces_multi(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                                       const int32_t *species, double *E, double *dEdrr, int32_t flags,
                                       void *stream) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!E) return ctx_fail(ctx, ACE_ERR_INVALID, "E is NULL");
  if (ctx->nprop < 1) return ctx_fail(ctx, ACE_ERR_INVALID, "no multi-property coefficients set");
  const bool din = flags & ACE_INPUTS_ON_DEVICE;
  if (din && dEdrr && !(flags & ACE_OUTPUTS_ON_DEVICE))
    return ctx_fail(ctx, ACE_ERR_INVALID, "host gradient output needs host inputs (the size is unknown)");
  int64_t nNbr = 0;
  if (!din) nNbr = offsets ? offsets[nEnv] : 0;
  else if (dEdrr && nEnv > 0) {
    ACE_CUDA(cudaSetDevice(ctx->device));
    ACE_CUDA(cudaMemcpy(&nNbr, offsets + nEnv, sizeof(int64_t), cudaMemcpyDeviceToHost));
  }
  const int np = ctx->nprop;
  const size_t csz = (ctx->prec == ACE_PREC_FP64 || ctx->prec == ACE_PREC_FP32X2) ? 8 : 4;
  const size_t per = (ctx->cplx ? 2 : 1) * ctx->ik.size() * csz;
  // real coefficient sets follow the context's schedule choice; complex ones
  // always run the item kernels
  if (!ctx->use_items && !ctx->cplx)
    return ctx_fail(ctx, ACE_ERR_UNSUPPORTED, "multi-property models need the item schedule");
  std::vector<std::pair<void *, size_t>> outs = {{E, (size_t)np * nEnv * sizeof(double)},
                                                 {dEdrr, (size_t)np * nNbr * 3 * sizeof(double)}};
  return drive(ctx, nEnv, offsets, rr, species, flags, stream, outs,
               [&](const int64_t *o, const double *x, const int32_t *s, std::vector<void *> &d, cudaStream_t st) {
                 for (int p = 0; p < np; ++p) {
                   const double c0 = ctx->has_const ? ctx->ctilde_multi[(size_t)p * ctx->nAA] : 0.0;
                   double *Ep = (double *)d[0] + (size_t)p * nEnv;
                   double *Gp = d[1] ? (double *)d[1] + (size_t)p * nNbr * 3 : nullptr;
                   int rc = launch_energy_forces(ctx, nEnv, o, x, s, Ep, Gp, st, (char *)ctx->d_ic_multi + p * per, c0,
                                                 ctx->cplx);
                   if (rc) return rc;
                 }
                 return (int)ACE_OK;
               });
}

extern "C" int ace_energy(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                          const int32_t *species, double *E, int32_t flags, void *stream) {
  return ace_energy_forces(ctx, nEnv, offsets, rr, species, E, nullptr, flags, stream);
}

extern "C" int ace_basis(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                         const int32_t *species, double *B, double *dB, int32_t flags, void *stream) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!B) return ctx_fail(ctx, ACE_ERR_INVALID, "B is NULL");
  if (ctx->nB == 0) return ctx_fail(ctx, ACE_ERR_INVALID, "spec has no U");
  if (dB && (flags & ACE_INPUTS_ON_DEVICE))
    return ctx_fail(ctx, ACE_ERR_INVALID, "dB needs host inputs (the size is unknown)");
  int64_t nNbr = (flags & ACE_INPUTS_ON_DEVICE) ? 0 : (offsets ? offsets[nEnv] : 0);
  std::vector<std::pair<void *, size_t>> outs = {{B, (size_t)nEnv * ctx->nB * sizeof(double)},
                                                 {dB, (size_t)nNbr * ctx->nB * 3 * sizeof(double)}};
  return drive(ctx, nEnv, offsets, rr, species, flags, stream, outs,
               [&](const int64_t *o, const double *x, const int32_t *s, std::vector<void *> &d, cudaStream_t st) {
                 int rc = launch_basis(ctx, nEnv, o, x, s, (double *)d[0], nullptr, st);
                 if (rc || !dB) return rc;
                 return launch_dbasis(ctx, nEnv, o, offsets, x, s, (double *)d[1], st);
               });
}

extern "C" int ace_adjoint_eval_d(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                                  const int32_t *species, const double *w, double *out, int32_t flags,
                                  void *stream) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!out || !w) return ctx_fail(ctx, ACE_ERR_INVALID, "w or out is NULL");
  if (ctx->nB == 0) return ctx_fail(ctx, ACE_ERR_INVALID, "spec has no U");
  const bool din = flags & ACE_INPUTS_ON_DEVICE;
  const double *d_w = w;
  if (!din) {
    // host weights: stage them next to the positions (3 per neighbour)
    const int64_t nNbr = offsets ? offsets[nEnv] : 0;
    const size_t bytes = std::max<int64_t>(nNbr, 1) * 3 * sizeof(double);
    ACE_CUDA(cudaSetDevice(ctx->device));
    if (bytes > ctx->wstage_bytes) {
      if (ctx->d_wstage) { cudaFree(ctx->d_wstage); ctx->d_wstage = nullptr; ctx->wstage_bytes = 0; }
      if (cudaMalloc(&ctx->d_wstage, bytes) != cudaSuccess) return ctx_fail(ctx, ACE_ERR_ALLOC, "staging allocation failed");
      ctx->wstage_bytes = bytes;
    }
    if (nNbr > 0)
      ACE_CUDA(cudaMemcpyAsync(ctx->d_wstage, w, nNbr * 3 * sizeof(double), cudaMemcpyHostToDevice, (cudaStream_t)stream));
    d_w = (const double *)ctx->d_wstage;
  }
  std::vector<std::pair<void *, size_t>> outs = {{out, (size_t)nEnv * ctx->nB * sizeof(double)}};
  return drive(ctx, nEnv, offsets, rr, species, flags, stream, outs,
               [&](const int64_t *o, const double *x, const int32_t *s, std::vector<void *> &d, cudaStream_t st) {
                 return launch_adjoint_eval_d(ctx, nEnv, o, nullptr, x, s, d_w, (double *)d[0], st);
               });
}

// Autotuner: times the energy/force kernel on the caller's batch (device
// pointers) for each candidate (correlation algorithm x shared-region size)
// and keeps the fastest.  Returns the chosen configuration in *choice
// (region_kb + 1000 * use_items) when choice is not NULL.
extern "C" int ace_autotune(ace_ctx *ctx, int64_t nEnv, const int64_t *offsets, const double *rr,
                            const int32_t *species, double *E, double *dEdrr, int32_t reps, void *stream,
                            int32_t *choice) {
  if (!ctx) return ACE_ERR_INVALID;
  if (!offsets || !rr || !E || nEnv < 1) return ctx_fail(ctx, ACE_ERR_INVALID, "autotune needs a non-empty device batch");
  if (input_species(ctx) > 1 && !species) return ctx_fail(ctx, ACE_ERR_INVALID, "species required for a multi-species spec");
  ACE_CUDA(cudaSetDevice(ctx->device));
  cudaStream_t st = (cudaStream_t)stream;
  const int regions[] = {16, 24, 32, 40, 48, 64};
  // candidates: the task schedule (orders >= 3) at its default and its high
  // occupancy, the item runs and, except for the compensated form (item
  // family only), the trie walk
  const int variants[] = {3, 2, 1, 0};
  const int nvariants = ctx->comp ? 3 : 4;
  float best = 1e30f;
  int best_region = ctx->region_kb;
  int best_variant = ctx->use_tasks ? (ctx->task_high ? 3 : 2) : ctx->use_items ? 1 : 0;
  cudaEvent_t e0, e1;
  ACE_CUDA(cudaEventCreate(&e0));
  ACE_CUDA(cudaEventCreate(&e1));
  reps = std::max(1, std::min(reps, 20));
  for (int vi = 0; vi < nvariants; ++vi) {
    const int variant = variants[vi];
    if (variant >= 2 && !ctx->has_tasks) continue;
    for (int reg : regions) {
      ctx->use_tasks = variant >= 2;
      ctx->task_high = variant == 3;
      ctx->use_items = variant >= 1;
      ctx->region_kb = reg;
      if (kernels_prepare(ctx) != ACE_OK) continue;
      const int32_t *sp = input_species(ctx) > 1 ? species : nullptr;
      int rc = launch_energy_forces(ctx, nEnv, offsets, rr, sp, E, dEdrr, st);  // warm-up
      if (rc) continue;
      // a candidate counts only when its launches and the timing succeeded
      bool timed = cudaEventRecord(e0, st) == cudaSuccess;
      for (int r = 0; r < reps && timed; ++r)
        timed = launch_energy_forces(ctx, nEnv, offsets, rr, sp, E, dEdrr, st) == ACE_OK;
      timed = timed && cudaEventRecord(e1, st) == cudaSuccess && cudaEventSynchronize(e1) == cudaSuccess;
      float ms = 0.f;
      timed = timed && cudaEventElapsedTime(&ms, e0, e1) == cudaSuccess;
      if (timed && cudaGetLastError() == cudaSuccess && ms < best) { best = ms; best_region = reg; best_variant = variant; }
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  ctx->use_tasks = best_variant >= 2;
  ctx->task_high = best_variant == 3;
  ctx->use_items = best_variant >= 1;
  ctx->region_kb = best_region;
  int rc = kernels_prepare(ctx);
  if (rc) return rc;
  if (choice) *choice = best_region + 1000 * best_variant;
  return read_status(ctx, st);
}

extern "C" int ace_sync(ace_ctx *ctx) {
  if (!ctx) return ACE_ERR_INVALID;
  ACE_CUDA(cudaSetDevice(ctx->device));
  ACE_CUDA(cudaDeviceSynchronize());
  return read_status(ctx, 0);
}

extern "C" int ace_get_spec_sizes(const ace_ctx *ctx, int64_t *sizes) {
  if (!ctx || !sizes) return ACE_ERR_INVALID;
  sizes[0] = ctx->nA; sizes[1] = ctx->nAA; sizes[2] = ctx->nB; sizes[3] = ctx->maxord;
  return ACE_OK;
}

extern "C" const char *ace_last_error_string(const ace_ctx *ctx) {
  return ctx ? ctx->err.c_str() : g_create_error.c_str();
}

extern "C" int64_t ace_launch_count(const ace_ctx *ctx) { return ctx ? ctx->launches : 0; }
