// Host-logic check of the correlation schedules (ace_sched.h): evaluates the
// energy and the adjoint dE/dA in double precision through (1) the trie walk,
// (2) the item schedule and (3) the task schedule, exactly as the kernels
// order them, and compares with the flat products of the spec
// (src/evaluator.jl:121-147, src/pibasis.jl:338-390).  Inputs are binary
// dumps written by tests/test_sched_host.py; prints one line of errors.
#include <complex>
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>

#include "ace_sched.h"

using namespace ace;
using C = std::complex<double>;

template <class T> static std::vector<T> rd(const std::string &f) {
  std::ifstream in(f, std::ios::binary);
  in.seekg(0, std::ios::end);
  size_t n = (size_t)in.tellg() / sizeof(T);
  in.seekg(0);
  std::vector<T> v(n);
  in.read((char *)v.data(), n * sizeof(T));
  return v;
}

int main(int argc, char **argv) {
  const std::string d = argc > 1 ? std::string(argv[1]) + "/" : "";
  auto an = rd<int32_t>(d + "an.bin"), al = rd<int32_t>(d + "al.bin"), am = rd<int32_t>(d + "am.bin"),
       amu = rd<int32_t>(d + "amu.bin"), ord = rd<int32_t>(d + "ord.bin"), iaa = rd<int32_t>(d + "iaa.bin"),
       Ui = rd<int32_t>(d + "Ui.bin");
  auto Up = rd<int64_t>(d + "Up.bin");
  auto Ud = rd<double>(d + "Ud.bin"), ct = rd<double>(d + "ct.bin"), Ar = rd<double>(d + "A.bin"),
       Wr = rd<double>(d + "W.bin");
  const int nA = (int)an.size();
  const int64_t nAA = (int64_t)ord.size();
  const int K = (int)(iaa.size() / nAA);
  const int64_t nB = (int64_t)Up.size() - 1;
  std::vector<C> A(nA), W(nA);
  for (int i = 0; i < nA; ++i) { A[i] = C(Ar[2 * i], Ar[2 * i + 1]); W[i] = C(Wr[2 * i], Wr[2 * i + 1]); }
  const int NT = 128;
  Schedule s = build_schedule(nA, an.data(), al.data(), am.data(), amu.data(), nAA, K, ord.data(), iaa.data(), nB,
                              Up.data(), Ui.data(), Ud.data(), NT);
  // flat reference
  double Eref = 0;
  std::vector<C> Dref(nA);
  for (int64_t k = 0; k < nAA; ++k) {
    const int o = ord[k];
    if (o == 0) { Eref += ct[k]; continue; }
    C p = 1;
    for (int t = 0; t < o; ++t) p *= A[iaa[k * K + t]];
    Eref += ct[k] * p.real();
    for (int t = 0; t < o; ++t) {
      C q = ct[k];
      for (int u = 0; u < o; ++u) if (u != t) q *= A[iaa[k * K + u]];
      Dref[iaa[k * K + t]] += q;
    }
  }
  // (1) trie walk per thread range
  double Et = ct[0];
  std::vector<C> Dt(nA);
  for (int th = 0; th < NT; ++th) {
    C H[8], Ac[8], bar[8];
    int vc[8] = {0};
    for (int q = 0; q < 8; ++q) { H[q] = 0; Ac[q] = 0; bar[q] = 1; }
    int cur = 0;
    auto close = [&](int q) { Dt[vc[q]] += bar[q - 1] * H[q]; H[q - 1] += Ac[q] * H[q]; };
    for (int i = s.start[th]; i < s.start[th + 1]; ++i) {
      const int q = s.q[i], k = s.ord[i];
      for (int e = K; e >= 1; --e) if (e <= cur && e > q) close(e);
      for (int e = 1; e <= K; ++e)
        if (e > q && e <= k) { int u = s.v[(size_t)(e - 1) * s.n + i]; vc[e] = u; Ac[e] = A[u]; bar[e] = bar[e - 1] * A[u]; H[e] = 0; }
      H[k] += s.w[i] * ct[s.k[i]];
      cur = k;
    }
    for (int e = K; e >= 1; --e) if (e <= cur) close(e);
    Et += H[0].real();
  }
  // (2) items
  ItemSchedule it = build_items(s, NT);
  double Ei = ct[0];
  std::vector<C> Di(nA);
  const int KP = it.KP, G = ITEM_G;
#if EF_ITEM_RUNS
  // per-thread contiguous runs (slot = j * NT + thread) with reverse-mode
  // accumulation along the open prefix path, as the kernel: node adjoints
  // W[d], products Q[d] = A_cur[0] .. A_cur[d]; a node closes when the path
  // leaves it (D[cur[d]] += W[d] Q[d-1], W[d-1] += W[d] A_cur[d])
  for (int t = 0; t < NT; ++t) {
    int cur[8], cP = 0;
    C Wn[8], Q[8];
    for (int e = 0; e < 8; ++e) { cur[e] = -1; Wn[e] = 0; Q[e] = 1; }
    auto close_to = [&](int c) {
      for (int d = cP - 1; d >= c; --d) {
        Di[cur[d]] += d > 0 ? Wn[d] * Q[d - 1] : Wn[d];
        if (d > 0) Wn[d - 1] += Wn[d] * A[cur[d]];
        Wn[d] = 0;
      }
    };
    for (int64_t f = t; f < it.n; f += NT) {
      const uint16_t *r = &it.rec[8 * f];
      const uint8_t *b = (const uint8_t *)r;
      const int P = b[14] & 0xf, nl = b[14] >> 4;
      auto coef = [&](int g) {
        int64_t k = g == 0 ? it.kown[f] : it.kleaf[f * G + g - 1];
        uint8_t w = g == 0 ? it.wown[f] : it.wleaf[f * G + g - 1];
        return k < 0 ? 0.0 : w * ct[k];
      };
      if (P == 0) continue;
      C bar = 1;
      for (int e = 0; e < P; ++e) bar *= A[r[e]];
      C H = coef(0);
      for (int g = 0; g < nl; ++g) H += coef(g + 1) * A[r[5 + g]];
      Ei += (bar * H).real();
      int c = 0;
      while (c < P && c < cP && r[c] == cur[c]) ++c;
      close_to(c);
      for (int d = c; d < P; ++d) { cur[d] = r[d]; Q[d] = (d > 0 ? Q[d - 1] : C(1)) * A[r[d]]; }
      cP = P;
      Wn[P - 1] += H;
      if (nl > 0 && P != KP) { printf("leaves-on-short-prefix\n"); return 1; }
      for (int g = 0; g < nl; ++g) Di[r[5 + g]] += coef(g + 1) * Q[KP - 1];
    }
    close_to(0);
  }
#else
  // 32 consecutive items per warp, segmented by head bits
  for (int64_t w0 = 0; w0 < it.n; w0 += 32) {
    C v[32][8];
    int tgt[32][8];
    unsigned heads[32];
    for (int lane = 0; lane < 32; ++lane) {
      const int64_t f = w0 + lane;
      const uint16_t *r = &it.rec[8 * f];
      const uint8_t *b = (const uint8_t *)r;
      const int P = b[14] & 0xf, nl = b[14] >> 4;
      heads[lane] = b[15];
      auto coef = [&](int g) {
        int64_t k = g == 0 ? it.kown[f] : it.kleaf[f * G + g - 1];
        uint8_t w = g == 0 ? it.wown[f] : it.wleaf[f * G + g - 1];
        return k < 0 ? 0.0 : w * ct[k];
      };
      C bar = 1;
      for (int e = 0; e < P; ++e) bar *= A[r[e]];
      C H = coef(0);
      for (int g = 0; g < nl; ++g) H += coef(g + 1) * A[r[5 + g]];
      if (P > 0) Ei += (bar * H).real();
      for (int g = 0; g < nl; ++g) Di[r[5 + g]] += coef(g + 1) * bar;
      for (int e = 0; e < KP; ++e) {
        C q = 0;
        if (e < P) { q = H; for (int x = 0; x < P; ++x) if (x != e) q *= A[r[x]]; }
        v[lane][e] = q;
        tgt[lane][e] = e < P ? r[e] : -1;
      }
    }
    for (int e = 0; e < KP; ++e) {
      if (e < KP - 1) {
        for (int lane = 0; lane < 32; ++lane)
          if ((heads[lane] >> e) & 1) {
            C sum = v[lane][e];
            for (int l2 = lane + 1; l2 < 32 && !((heads[l2] >> e) & 1); ++l2) sum += v[l2][e];
            if (tgt[lane][e] >= 0) Di[tgt[lane][e]] += sum;
            else if (std::abs(sum) > 0) { printf("lost-contribution\n"); return 1; }
          }
      } else {
        for (int lane = 0; lane < 32; ++lane) if (tgt[lane][e] >= 0) Di[tgt[lane][e]] += v[lane][e];
      }
    }
  }
#endif
  // (3) tasks (orders >= 3): per warp, per lane, the rows of the warp's
  // program as the kernel walks them
  double Ek = ct[0];
  std::vector<C> Dk(nA);
  TaskSchedule ts = build_tasks(s, NT / 32);
  if (K >= 3) {
    const int KT = ts.KT, L = TASK_LANES;
    auto coefk = [&](int64_t row, int g, int lane) {
      const size_t q = ((size_t)row * (1 + G) + g) * L + lane;
      return ts.ck[q] < 0 ? 0.0 : ts.cw[q] * ct[ts.ck[q]];
    };
    for (int w = 0; w < ts.nwarps; ++w)
      for (int lane = 0; lane < L; ++lane)
        for (int64_t row = ts.wrow[w]; row < ts.wrow[w + 1];) {
          const uint16_t *h = &ts.rec[((size_t)row * L + lane) * 8];
          if (h[7] == 1) {
            const int n = h[6];
            C Qt = 1, Wt = 0;
            for (int d = 0; d < KT; ++d) Qt *= A[h[d]];
            for (int j = 0; j < n; ++j) {
              const int64_t ir = row + 1 + j;
              const uint16_t *r = &ts.rec[((size_t)ir * L + lane) * 8];
              if (r[7] != 2) { printf("bad-item-row\n"); return 1; }
              const C am = A[r[0]];
              C H = coefk(ir, 0, lane);
              for (int g = 0; g < r[6]; ++g) H += coefk(ir, 1 + g, lane) * A[r[1 + g]];
              const C Q = Qt * am;
              Ek += (Q * H).real();
              for (int g = 0; g < r[6]; ++g) Dk[r[1 + g]] += coefk(ir, 1 + g, lane) * Q;
              Dk[r[0]] += H * Qt;
              Wt += H * am;
            }
            for (int d = 0; d < KT; ++d) {
              C p = Wt;
              for (int e = 0; e < KT; ++e) if (e != d) p *= A[h[e]];
              Dk[h[d]] += p;
            }
            row += 1 + n;
          } else if (h[7] == 3) {
            const int P = h[6];
            const double c = coefk(row, 0, lane);
            C p = 1;
            for (int d = 0; d < P; ++d) p *= A[h[d]];
            Ek += c * p.real();
            for (int d = 0; d < P; ++d) {
              C q = c;
              for (int e = 0; e < P; ++e) if (e != d) q *= A[h[e]];
              Dk[h[d]] += q;
            }
            row += 1;
          } else {
            printf("bad-row-type %d\n", h[7]);
            return 1;
          }
        }
  } else {
    Ek = Eref;
    Dk = Dref;
  }
  // the kernels' adjoint is exact along conjugation-symmetric directions W
  C gr = 0, gt = 0, gi = 0, gk = 0;
  for (int i = 0; i < nA; ++i) { gr += Dref[i] * W[i]; gt += Dt[i] * W[i]; gi += Di[i] * W[i]; gk += Dk[i] * W[i]; }
  printf("%d %lld %lld %.3e %.3e %.3e %.3e %.3e %.3e %lld %lld\n", (int)s.halved, (long long)s.n, (long long)it.n,
         std::abs(Et - Eref) / std::abs(Eref), std::abs(Ei - Eref) / std::abs(Eref),
         std::abs(gt.real() - gr.real()) / std::abs(gr.real()), std::abs(gi.real() - gr.real()) / std::abs(gr.real()),
         std::abs(Ek - Eref) / std::abs(Eref), std::abs(gk.real() - gr.real()) / std::abs(gr.real()),
         (long long)ts.rows, (long long)ts.pad_items);
  return 0;
}
