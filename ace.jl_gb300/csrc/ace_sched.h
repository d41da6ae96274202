// ace_sched.h -- host-side preparation of the correlation (AA) evaluation
// schedule consumed by the trie kernel.
//
// The reference evaluates each AA function as a flat product
// (src/evaluator.jl:137-142, src/pibasis.jl:265-275).  Here the functions are
// visited in lexicographic order of their (descending) index tuples, so that
// functions sharing a prefix (v1, ..., vd) are adjacent: the kernel keeps the
// prefix products and Horner partial sums of the current path in registers,
// which is the recursive product evaluation of src/grapheval.jl:80-278
// restricted to prefix splits.
//
// Conjugation symmetry: for real positions A_{n,l,-m} = (-1)^m conj(A_{n,l,m}),
// so AA of the m-reversed tuple is the complex conjugate (sum m = 0), and the
// invariant coupling gives both the same c~.  Only one function of each such
// pair is kept, with weight 2; the same weights give the correct adjoint for
// the forces (the partner's contribution to Re(dAco . dA) is identical).  The
// halving is used only if every partner exists and U has identical columns
// for both partners.
#pragma once
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <map>
#include <numeric>
#include <queue>
#include <tuple>
#include <utility>
#include <vector>

namespace ace {

struct Schedule {
  int K = 0;                       // maximum order
  int64_t n = 0;                   // scheduled functions (order >= 1)
  std::vector<uint16_t> v;         // [K][n] indices (descending within a function)
  std::vector<uint8_t> ord;        // [n]
  std::vector<uint8_t> q;          // [n] common prefix length with the previous function
  std::vector<int32_t> k;          // [n] index of the AA function in the spec
  std::vector<uint8_t> w;          // [n] weight (1, or 2 for a conjugate pair)
  std::vector<int32_t> start;      // [nthreads + 1] per-thread ranges
  bool halved = false;
  int64_t nodes = 0;               // trie nodes opened (for accounting)
  // when halved: the m-reversed partner of every AA function and (-1)^{sum m}
  // (AA_partner = (-1)^{sum m} conj(AA)), for merging complex coefficients
  std::vector<int64_t> partner;
  std::vector<int8_t> msign;
};

// Lexicographic key of a descending index tuple of length <= 6: (v_j + 1) in
// 16-bit fields from the most significant end and 0 past the tuple's end, so
// keys order like std::vector comparison (a proper prefix sorts first).
struct TupleKey {
  uint64_t hi = 0, lo = 0;  // fields 0-1 in hi, 2-5 in lo
  bool operator<(const TupleKey &o) const { return hi < o.hi || (hi == o.hi && lo < o.lo); }
  bool operator==(const TupleKey &o) const { return hi == o.hi && lo == o.lo; }
};

inline TupleKey tuple_key(const int32_t *t, int o) {
  TupleKey key;
  for (int j = 0; j < 6; ++j) {
    const uint64_t f = j < o ? (uint64_t)(uint16_t)(t[j] + 1) : 0u;
    if (j < 2) key.hi = (key.hi << 16) | f;
    else key.lo = (key.lo << 16) | f;
  }
  return key;
}

inline Schedule build_schedule(int nA, const int32_t *a_n, const int32_t *a_l, const int32_t *a_m,
                               const int32_t *a_mu, int64_t nAA, int K, const int32_t *orders,
                               const int32_t *iAA2iA, int64_t nB, const int64_t *U_indptr,
                               const int32_t *U_indices, const double *U_data, int nthreads) {
  Schedule s;
  s.K = K;
  // ---- partner A indices (m -> -m)
  std::map<std::tuple<int, int, int, int>, int> aidx;
  for (int i = 0; i < nA; ++i) aidx[{a_mu ? a_mu[i] : 0, a_n[i], a_l[i], a_m[i]}] = i;
  std::vector<int> partner(nA, -1);
  bool ok = true;
  for (int i = 0; i < nA; ++i) {
    auto it = aidx.find({a_mu ? a_mu[i] : 0, a_n[i], a_l[i], -a_m[i]});
    if (it == aidx.end()) { ok = false; break; }
    partner[i] = it->second;
  }
  // ---- partner AA functions: the keys of all tuples and of their partner
  // tuples, both sorted, joined in one merge (for a repeated tuple the last
  // function, as a map would give)
  typedef std::pair<TupleKey, int64_t> KeyedK;
  auto by_key = [](const KeyedK &a, const KeyedK &b) {
    return a.first < b.first || (a.first == b.first && a.second < b.second);
  };
  std::vector<KeyedK> keyed((size_t)nAA);
  for (int64_t k = 0; k < nAA; ++k) keyed[k] = {tuple_key(iAA2iA + k * K, orders[k]), k};
  std::sort(keyed.begin(), keyed.end(), by_key);
  std::vector<int64_t> pk(nAA, -1);
  if (ok) {
    std::vector<KeyedK> pkeyed((size_t)nAA);
    int32_t t[8];
    for (int64_t k = 0; k < nAA; ++k) {
      const int o = orders[k];
      for (int j = 0; j < o; ++j) t[j] = partner[iAA2iA[k * K + j]];
      for (int a = 1; a < o; ++a) {  // descending insertion sort (o <= 6)
        const int32_t x = t[a];
        int b = a - 1;
        while (b >= 0 && t[b] < x) { t[b + 1] = t[b]; --b; }
        t[b + 1] = x;
      }
      pkeyed[k] = {tuple_key(t, o), k};
    }
    std::sort(pkeyed.begin(), pkeyed.end(), by_key);
    size_t a = 0;
    for (size_t i = 0; i < pkeyed.size(); ++i) {
      const TupleKey &key = pkeyed[i].first;
      while (a < keyed.size() && keyed[a].first < key) ++a;
      size_t e = a;
      while (e < keyed.size() && keyed[e].first == key) ++e;
      if (e == a) { ok = false; break; }
      pk[pkeyed[i].second] = keyed[e - 1].second;
    }
  }
  std::vector<std::pair<TupleKey, int64_t>>().swap(keyed);
  // ---- U columns of partners must agree (then c~ agrees for every c):
  // columns of U (CSC, rows ascending) by counting sort
  if (ok && nB > 0) {
    const int64_t nnz = U_indptr[nB];
    std::vector<int64_t> cptr(nAA + 1, 0);
    for (int64_t j = 0; j < nnz; ++j) cptr[U_indices[j] + 1]++;
    for (int64_t k = 0; k < nAA; ++k) cptr[k + 1] += cptr[k];
    std::vector<int64_t> crow(nnz), fill(cptr.begin(), cptr.end() - 1);
    std::vector<double> cval(nnz);
    for (int64_t b = 0; b < nB; ++b)
      for (int64_t j = U_indptr[b]; j < U_indptr[b + 1]; ++j) {
        const int64_t q = fill[U_indices[j]]++;
        crow[q] = b;
        cval[q] = U_data[j];
      }
    for (int64_t k = 0; k < nAA && ok; ++k) {
      const int64_t a0 = cptr[k], na = cptr[k + 1] - a0, b0 = cptr[pk[k]], nb = cptr[pk[k] + 1] - b0;
      if (na != nb) { ok = false; break; }
      for (int64_t j = 0; j < na; ++j)
        if (crow[a0 + j] != crow[b0 + j] ||
            std::fabs(cval[a0 + j] - cval[b0 + j]) > 1e-12 * (1.0 + std::fabs(cval[a0 + j]))) {
          ok = false; break;
        }
    }
  }
  s.halved = ok;
  if (ok) {
    s.partner = pk;
    s.msign.resize(nAA);
    for (int64_t k = 0; k < nAA; ++k) {
      int msum = 0;
      for (int j = 0; j < orders[k]; ++j) msum += a_m[iAA2iA[k * K + j]];
      s.msign[k] = (msum % 2 == 0) ? 1 : -1;
    }
  }
  // ---- kept functions (order >= 1)
  std::vector<int64_t> keep;
  std::vector<uint8_t> wts;
  for (int64_t k = 0; k < nAA; ++k) {
    if (orders[k] == 0) continue;
    if (ok) {
      if (pk[k] == k) { keep.push_back(k); wts.push_back(1); }
      else if (pk[k] > k) { keep.push_back(k); wts.push_back(2); }
    } else {
      keep.push_back(k); wts.push_back(1);
    }
  }
  // ---- lexicographic order of the descending tuples (prefix first)
  std::vector<std::pair<TupleKey, size_t>> order(keep.size());
  for (size_t i = 0; i < keep.size(); ++i) order[i] = {tuple_key(iAA2iA + keep[i] * K, orders[keep[i]]), i};
  std::stable_sort(order.begin(), order.end(), [](const std::pair<TupleKey, size_t> &a, const std::pair<TupleKey, size_t> &b) {
    return a.first < b.first;
  });
  s.n = (int64_t)keep.size();
  s.v.assign((size_t)K * s.n, 0);
  s.ord.resize(s.n); s.q.resize(s.n); s.k.resize(s.n); s.w.resize(s.n);
  const int32_t *prev = nullptr;
  int prev_o = 0;
  for (int64_t i = 0; i < s.n; ++i) {
    const size_t pi = order[i].second;
    const int64_t k = keep[pi];
    const int o = orders[k];
    const int32_t *t = iAA2iA + k * K;
    s.ord[i] = (uint8_t)o;
    s.k[i] = (int32_t)k;
    s.w[i] = wts[pi];
    for (int j = 0; j < o; ++j) s.v[(size_t)j * s.n + i] = (uint16_t)t[j];
    int qq = 0;
    if (prev)
      while (qq < std::min(prev_o, o) && prev[qq] == t[qq]) ++qq;
    s.q[i] = (uint8_t)qq;
    prev = t;
    prev_o = o;
  }
  // ---- contiguous ranges of (nearly) equal length, one per thread
  s.start.assign(nthreads + 1, 0);
  for (int t = 0; t <= nthreads; ++t) s.start[t] = (int32_t)((s.n * (int64_t)t) / nthreads);
  // a range starts from an empty path
  for (int t = 0; t < nthreads; ++t)
    if (s.start[t] < s.n) s.q[s.start[t]] = 0;
  for (int64_t i = 0; i < s.n; ++i) s.nodes += s.ord[i] - s.q[i];
  return s;
}

// Thread-interleaved records: slot (j * nthreads + t) holds the j-th function
// of thread t's range, so that the lanes of a warp read adjacent 16-byte
// records.  Record: v[0..5] (uint16), ord (uint8), q (uint8), 2 bytes pad;
// ord == 0 marks an empty slot.  perm[slot] is the schedule index (-1: empty).
struct Interleaved {
  int64_t len = 0;                 // slots per thread
  std::vector<uint16_t> rec;       // [len * nthreads * 8]
  std::vector<int64_t> perm;       // [len * nthreads]
};

inline Interleaved interleave(const Schedule &s, int nthreads) {
  Interleaved r;
  int64_t mx = 0;
  for (int t = 0; t < nthreads; ++t) mx = std::max<int64_t>(mx, s.start[t + 1] - s.start[t]);
  r.len = mx;
  r.rec.assign((size_t)mx * nthreads * 8, 0);
  r.perm.assign((size_t)mx * nthreads, -1);
  // slot order (j outer): the writes are sequential
  for (int64_t j = 0; j < mx; ++j)
    for (int t = 0; t < nthreads; ++t) {
      const int64_t i = s.start[t] + j;
      if (i >= s.start[t + 1]) continue;
      const size_t slot = (size_t)j * nthreads + t;
      uint16_t *rc = &r.rec[8 * slot];
      for (int d = 0; d < s.K && d < 6; ++d) rc[d] = s.v[(size_t)d * s.n + i];
      rc[6] = (uint16_t)(s.ord[i] | (s.q[i] << 8));
      r.perm[slot] = i;
    }
  return r;
}

// ----------------------------------------------------------------------------
// Item schedule (uniform per-lane work).  A depth-(K-1) prefix p = (v1..v_{K-1})
// together with up to G of its leaves (v1..v_{K-1}, u) is one item; a prefix
// with more leaves is split into several items (every quantity an item
// contributes is linear in its leaves, so the split is exact).  The
// coefficient of the prefix function itself, if p is a function, rides on
// the prefix's first item.  Functions of order < K-1 are items with no
// leaves.  Items are sorted lexicographically by prefix (full-length prefixes
// first), so items sharing a prefix (v1..vd) are adjacent.  With the default
// layout (EF_ITEM_RUNS = 1) each thread takes a contiguous run of the sorted
// items and accumulates the prefix adjoints in reverse mode along the run
// (per trie node of its open path); with EF_ITEM_RUNS = 0 a warp processes
// 32 consecutive items and reduces the adjoint contributions to shared
// targets with segmented shuffles, for which `head` bit d marks the first
// item of a run of equal (v1..v_{d+1}) within its warp.
//
// Record (16 bytes): idx[0..4] prefix (uint16), idx[5..6] leaves, byte 14 =
// P | nleaf << 4, byte 15 = head bits.  P == 0 marks padding.
static constexpr int ITEM_G = 2;

// item layout: 1 (default) = per-thread contiguous runs with the prefix
// adjoints accumulated in registers along the run; 0 = uniform stride with
// warp-segmented prefix reductions using the head bits
#ifndef EF_ITEM_RUNS
#define EF_ITEM_RUNS 1
#endif

struct ItemSchedule {
  int K = 0, KP = 0;               // max order, max prefix length (K - 1)
  int64_t n = 0;                   // items, padded to a multiple of the block size
  std::vector<uint16_t> rec;       // [n * 8]
  std::vector<int64_t> kown;       // [n] AA index of the prefix function (-1: none)
  std::vector<int64_t> kleaf;      // [n * G] AA index of each leaf (-1: none)
  std::vector<uint8_t> wown, wleaf;
};

inline ItemSchedule build_items(const Schedule &s, int nthreads) {
  ItemSchedule it;
  const int K = s.K;
  it.K = K;
  it.KP = K > 1 ? K - 1 : 1;
  const int KP = it.KP;
  struct Item {
    int P = 0, nl = 0;
    int pre[6] = {0, 0, 0, 0, 0, 0};
    int64_t kown = -1;
    uint8_t wown = 0;
    int leaf[ITEM_G] = {};
    int64_t kleaf[ITEM_G] = {};
    uint8_t wleaf[ITEM_G] = {};
  };
  // One pass over the functions in lexicographic order: the functions with a
  // prefix p of length K-1 (p itself first, then its extensions) are
  // adjacent, so each prefix's items are formed where its first function
  // appears; shorter functions are collected in order and appended.
  std::vector<Item> items, shorts;
  int cur[6] = {0, 0, 0, 0, 0, 0};
  bool have = false;
  size_t cur_first = 0;
  auto vat = [&](int64_t i, int j) { return (int)s.v[(size_t)j * s.n + i]; };
  auto open_group = [&](int64_t i) {  // the group of prefix v[0..KP) of function i
    bool same = have;
    for (int j = 0; j < KP && same; ++j) same = cur[j] == vat(i, j);
    if (!same) {
      Item x;
      x.P = KP;
      for (int j = 0; j < KP; ++j) cur[j] = x.pre[j] = vat(i, j);
      items.push_back(x);
      cur_first = items.size() - 1;
      have = true;
    }
  };
  for (int64_t i = 0; i < s.n; ++i) {
    const int o = s.ord[i];
    if (K > 1 && o == K) {
      open_group(i);
      if (items.back().nl == ITEM_G) {
        Item x;
        x.P = KP;
        for (int j = 0; j < KP; ++j) x.pre[j] = cur[j];
        items.push_back(x);
      }
      Item &b = items.back();
      b.leaf[b.nl] = vat(i, K - 1);
      b.kleaf[b.nl] = s.k[i];
      b.wleaf[b.nl] = s.w[i];
      ++b.nl;
    } else if (o == KP) {
      open_group(i);
      items[cur_first].kown = s.k[i];
      items[cur_first].wown = s.w[i];
    } else {
      Item x;
      x.P = o;
      for (int j = 0; j < o; ++j) x.pre[j] = vat(i, j);
      x.kown = s.k[i];
      x.wown = s.w[i];
      shorts.push_back(x);
    }
  }
  items.insert(items.end(), shorts.begin(), shorts.end());
  const int64_t n0 = (int64_t)items.size();
  it.n = ((n0 + nthreads - 1) / nthreads) * nthreads;
  if (it.n == 0) it.n = nthreads;
#if EF_ITEM_RUNS
  // each thread takes a contiguous run of the sorted items, interleaved
  // (slot = j * nthreads + thread): consecutive items of a thread share
  // prefixes, so the kernel keeps their prefix adjoints in registers
  {
    const int64_t R = it.n / nthreads;
    std::vector<Item> laid(it.n);
    for (int64_t i = 0; i < n0; ++i) laid[(i % R) * nthreads + i / R] = items[i];
    items.swap(laid);
  }
  const int64_t nfill = it.n;
#else
  const int64_t nfill = n0;
#endif
  it.rec.assign((size_t)it.n * 8, 0);
  it.kown.assign(it.n, -1);
  it.kleaf.assign((size_t)it.n * ITEM_G, -1);
  it.wown.assign(it.n, 0);
  it.wleaf.assign((size_t)it.n * ITEM_G, 0);
  for (int64_t f = 0; f < nfill; ++f) {
    const Item &x = items[f];
    if (x.P == 0 && x.nl == 0 && x.kown < 0) continue;  // padding
    uint16_t *r = &it.rec[8 * f];
    const int P = x.P;
    for (int d = 0; d < P; ++d) r[d] = (uint16_t)x.pre[d];
    const int nl = x.nl;
    for (int g = 0; g < nl; ++g) {
      ((uint16_t *)r)[5 + g] = (uint16_t)x.leaf[g];
      it.kleaf[(size_t)f * ITEM_G + g] = x.kleaf[g];
      it.wleaf[(size_t)f * ITEM_G + g] = x.wleaf[g];
    }
    it.kown[f] = x.kown;
    it.wown[f] = x.wown;
    uint8_t heads = 0;
    for (int d = 0; d < KP; ++d) {
      bool head = (f % 32 == 0);
      if (!head) {
        const Item &y = items[f - 1];
        if (y.P != P || d >= P) head = true;
        else for (int e = 0; e <= d; ++e) if (y.pre[e] != x.pre[e]) { head = true; break; }
      }
      if (head) heads |= (uint8_t)(1u << d);
    }
    uint8_t *b = (uint8_t *)r;
    b[14] = (uint8_t)(P | (nl << 4));
    b[15] = heads;
  }
#if !EF_ITEM_RUNS
  for (int64_t f = n0; f < it.n; ++f) ((uint8_t *)&it.rec[8 * f])[15] = 0x1f;  // padding: own segments
#endif
  return it;
}

// ----------------------------------------------------------------------------
// Task schedule (orders K >= 3).  A task is a node of the prefix trie at depth
// KT - 1 (KT = K - 2): a prefix t = (v1..v_KT) and the full-length items
// below it, each item one more prefix index ("mid", v_{KT+1}), up to G
// leaves and the coefficient of the prefix function (t, mid) itself.  A lane
// evaluates a whole task: the task product Q_t = prod A_t once, for every
// item Q = Q_t A_mid, the energy Re(Q (c_own + sum_g c_g A_leaf_g)) and the
// adjoints (leaves: Q c_g; mid: H Q_t; the task's W += H A_mid), and at the
// end distributes W over the task prefix (D[t_d] += W prod_{d' != d} A_t_d').
// The same sums as the trie walk (src/pibasis.jl:338-390, grouped by node),
// with no open path carried from task to task.
//
// Tasks sorted by item count are grouped 32 at a time into warp "slots", so
// the lanes of a warp run tasks of (nearly) equal length in lockstep: a
// slot's length is its longest task's, shorter tasks end in zero-coefficient
// items, and the last slot is padded with zero-coefficient tasks; functions
// of order < K - 1 are "short" items, 32 of equal order per row, evaluated
// flat (product and local adjoints).  Slots are assigned to the warps of the
// CTA costliest first, each to the warp with the least work.
//
// Each warp runs its rows [wrow[w], wrow[w+1]); row r of lane l is record
// r * 32 + l (16 bytes, 8 uint16): a task header (type 1: t in [0..KT), the
// item count n in [6]), an item (type 2: mid in [0], leaves in [1..G],
// nl in [6]) or a short item (type 3: its indices in [0..P), P in [6]);
// [7] holds the type.  Coefficients: (1 + G) rows per record row,
// coefficient g of row r, lane l at ((r (1 + G) + g) 32 + l): an item's own
// coefficient and its leaves', a short item's in g = 0.
static constexpr int TASK_LANES = 32;

struct TaskSchedule {
  int K = 0, KT = 0, nwarps = 0;
  int64_t rows = 0;
  std::vector<int32_t> wrow;       // [nwarps + 1]
  std::vector<uint16_t> rec;       // [rows * 32 * 8]
  std::vector<int64_t> ck;         // [rows * (1 + G) * 32] AA index of each coefficient (-1: none)
  std::vector<uint8_t> cw;         // weights (1, or 2 for a conjugate pair)
  int64_t tasks = 0, items = 0, shorts = 0, pad_items = 0;
};

inline TaskSchedule build_tasks(const Schedule &s, int nwarps) {
  TaskSchedule ts;
  const int K = s.K, KP = K - 1, KT = K - 2, G = ITEM_G;
  ts.K = K;
  ts.KT = KT;
  ts.nwarps = nwarps;
  if (K < 3) return ts;
  auto vat = [&](int64_t i, int j) { return (int)s.v[(size_t)j * s.n + i]; };
  struct It { int mid; int nl; int leaf[ITEM_G]; int64_t kown; uint8_t wown; int64_t kl[ITEM_G]; uint8_t wl[ITEM_G]; };
  struct Task { int t[6]; std::vector<It> items; };
  struct Short { int P; int v[6]; int64_t k; uint8_t w; };
  std::vector<Task> tasks;
  std::vector<Short> shorts;
  // one pass in lexicographic order: the functions of a full prefix
  // (t, mid) -- the prefix function first, then its extensions -- are
  // adjacent, and so are the prefixes of a task
  int cur[6] = {-1, -1, -1, -1, -1, -1};
  bool have = false;
  auto open_item = [&](int64_t i) {
    bool same_task = have;
    for (int j = 0; j < KT && same_task; ++j) same_task = tasks.back().t[j] == vat(i, j);
    if (!same_task) {
      Task t;
      for (int j = 0; j < 6; ++j) t.t[j] = j < KT ? vat(i, j) : 0;
      tasks.push_back(t);
      have = true;
      cur[KT] = -1;
    }
    Task &t = tasks.back();
    const int mid = vat(i, KT);
    if (t.items.empty() || cur[KT] != mid || t.items.back().nl == G) {
      It x{};
      x.mid = mid;
      x.kown = -1;
      for (int g = 0; g < G; ++g) x.kl[g] = -1;
      // a repeated mid (more than G leaves) starts a new item without the
      // prefix function's coefficient
      t.items.push_back(x);
      cur[KT] = mid;
    }
  };
  for (int64_t i = 0; i < s.n; ++i) {
    const int o = s.ord[i];
    if (o == K) {
      open_item(i);
      It &x = tasks.back().items.back();
      x.leaf[x.nl] = vat(i, KP);
      x.kl[x.nl] = s.k[i];
      x.wl[x.nl] = s.w[i];
      ++x.nl;
    } else if (o == KP) {
      open_item(i);
      It &x = tasks.back().items.back();
      if (x.kown >= 0 || x.nl > 0) {  // (cannot happen in lexicographic order: the prefix sorts first)
        It y{};
        y.mid = x.mid;
        for (int g = 0; g < G; ++g) y.kl[g] = -1;
        tasks.back().items.push_back(y);
      }
      tasks.back().items.back().kown = s.k[i];
      tasks.back().items.back().wown = s.w[i];
    } else {
      Short sh{};
      sh.P = o;
      for (int j = 0; j < o; ++j) sh.v[j] = vat(i, j);
      sh.k = s.k[i];
      sh.w = s.w[i];
      shorts.push_back(sh);
    }
  }
  ts.tasks = (int64_t)tasks.size();
  ts.shorts = (int64_t)shorts.size();
  // slots: 32 tasks of equal item count, or 32 short items of equal order
  struct Slot { int kind; int n; std::vector<int> who; int64_t rows; };
  std::vector<Slot> slots;
  {
    // tasks by item count, longest first; 32 consecutive ones form a slot
    // whose length is its longest task's (shorter tasks end in
    // zero-coefficient items).  Tasks of equal length are taken in a
    // scrambled order: lexicographic neighbours share most of their A
    // indices, and 32 of them in one warp would serialise the adjoint's
    // shared-memory atomics on the same addresses.
    auto scramble = [](uint32_t x) {
      x ^= x >> 16; x *= 0x7feb352du; x ^= x >> 15; x *= 0x846ca68bu; x ^= x >> 16;
      return x;
    };
    std::vector<int> bylen(tasks.size());
    std::iota(bylen.begin(), bylen.end(), 0);
    std::stable_sort(bylen.begin(), bylen.end(), [&](int x, int y) {
      const size_t nx = tasks[x].items.size(), ny = tasks[y].items.size();
      return nx > ny || (nx == ny && scramble((uint32_t)x) < scramble((uint32_t)y));
    });
    for (size_t q = 0; q < bylen.size(); q += TASK_LANES) {
      Slot sl;
      sl.kind = 1;
      sl.n = (int)tasks[bylen[q]].items.size();
      for (size_t r = q; r < std::min(bylen.size(), q + TASK_LANES); ++r) {
        sl.who.push_back(bylen[r]);
        ts.items += (int64_t)tasks[bylen[r]].items.size();
      }
      sl.rows = 1 + sl.n;
      ts.pad_items += (int64_t)TASK_LANES * sl.n;
      slots.push_back(sl);
    }
    ts.pad_items -= ts.items;
    std::map<int, std::vector<int>> byord;
    for (int i = 0; i < (int)shorts.size(); ++i) byord[shorts[i].P].push_back(i);
    for (auto &kv : byord)
      std::stable_sort(kv.second.begin(), kv.second.end(),
                       [&](int x, int y) { return scramble((uint32_t)x) < scramble((uint32_t)y); });
    for (auto &kv : byord)
      for (size_t q = 0; q < kv.second.size(); q += TASK_LANES) {
        Slot sl;
        sl.kind = 3;
        sl.n = kv.first;
        for (size_t r = q; r < std::min(kv.second.size(), q + TASK_LANES); ++r) sl.who.push_back(kv.second[r]);
        sl.rows = 1;
        slots.push_back(sl);
      }
  }
  // balance: costliest slots first, each to the warp with the least work;
  // a task header (the task product and the distribution of its adjoint)
  // costs about three item rows
  auto cost = [&](const Slot &sl) { return sl.kind == 1 ? sl.rows + 2 : sl.rows; };
  std::vector<size_t> order(slots.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return cost(slots[x]) > cost(slots[y]); });
  std::vector<std::vector<size_t>> own(nwarps);
  std::vector<int64_t> load(nwarps, 0), nrows(nwarps, 0);
  for (size_t si : order) {
    int w = (int)(std::min_element(load.begin(), load.end()) - load.begin());
    own[w].push_back(si);
    load[w] += cost(slots[si]);
    nrows[w] += slots[si].rows;
  }
  ts.wrow.assign(nwarps + 1, 0);
  for (int w = 0; w < nwarps; ++w) ts.wrow[w + 1] = ts.wrow[w] + (int32_t)nrows[w];
  ts.rows = ts.wrow[nwarps];
  ts.rec.assign((size_t)ts.rows * TASK_LANES * 8, 0);
  ts.ck.assign((size_t)ts.rows * (1 + G) * TASK_LANES, -1);
  ts.cw.assign((size_t)ts.rows * (1 + G) * TASK_LANES, 0);
  auto recp = [&](int64_t row, int lane) { return &ts.rec[((size_t)row * TASK_LANES + lane) * 8]; };
  auto setc = [&](int64_t row, int g, int lane, int64_t k, uint8_t w) {
    const size_t q = ((size_t)row * (1 + G) + g) * TASK_LANES + lane;
    ts.ck[q] = k;
    ts.cw[q] = w;
  };
  for (int w = 0; w < nwarps; ++w) {
    int64_t row = ts.wrow[w];
    for (size_t si : own[w]) {
      const Slot &sl = slots[si];
      if (sl.kind == 1) {
        for (int lane = 0; lane < TASK_LANES; ++lane) {
          uint16_t *h = recp(row, lane);
          h[6] = (uint16_t)sl.n;
          h[7] = 1;
          for (int j = 0; j < sl.n; ++j) {
            uint16_t *r = recp(row + 1 + j, lane);
            r[6] = 0;
            r[7] = 2;
          }
          if (lane >= (int)sl.who.size()) continue;  // padding: index 0, no coefficients
          const Task &t = tasks[sl.who[lane]];
          for (int d = 0; d < KT; ++d) h[d] = (uint16_t)t.t[d];
          for (int j = 0; j < (int)t.items.size(); ++j) {
            const It &x = t.items[j];
            uint16_t *r = recp(row + 1 + j, lane);
            r[0] = (uint16_t)x.mid;
            for (int g = 0; g < x.nl; ++g) r[1 + g] = (uint16_t)x.leaf[g];
            r[6] = (uint16_t)x.nl;
            if (x.kown >= 0) setc(row + 1 + j, 0, lane, x.kown, x.wown);
            for (int g = 0; g < x.nl; ++g) setc(row + 1 + j, 1 + g, lane, x.kl[g], x.wl[g]);
          }
        }
      } else {
        for (int lane = 0; lane < TASK_LANES; ++lane) {
          uint16_t *r = recp(row, lane);
          r[6] = (uint16_t)sl.n;
          r[7] = 3;
          if (lane >= (int)sl.who.size()) continue;
          const Short &sh = shorts[sl.who[lane]];
          for (int d = 0; d < sh.P; ++d) r[d] = (uint16_t)sh.v[d];
          setc(row, 0, lane, sh.k, sh.w);
        }
      }
      row += sl.rows;
    }
  }
  return ts;
}

// Fused symmetric-basis table (B = U real(AA) without AA in memory).  U's
// rows are grouped into classes -- consecutive rows whose AA columns overlap
// (the rows of one (n, l)-class; different classes use disjoint AA
// functions) -- of at most UB_R rows.  Each AA function of a group is one
// entry: the kernel forms real(AA_k) once and adds U[b, k] real(AA_k) to the
// group's UB_R row accumulators.  With a halved schedule an AA function and
// its m-reversed partner (equal real parts for invariants) share one entry
// whose values are the sum of both U columns.  Groups are assigned to
// threads longest first, each to the least-loaded thread, and each thread's
// entries interleaved (slot = j * nthreads + thread).
// Record (16 bytes): x, y, z = A indices v0..v5 (uint16 pairs),
// w = b0 | ord << 24 | (r - 1) << 27 | last-of-group << 30 | valid << 31
// (b0 = the group's first row, r = its rows); values [slot][UB_R].
static constexpr int UB_R = 8;

struct URows {
  int64_t len = 0;                 // slots per thread
  std::vector<uint32_t> rec;       // [len * nthreads * 4]
  std::vector<double> val;         // [len * nthreads * UB_R]
};

inline URows build_urows(int64_t nB, const int64_t *Uptr, const int32_t *Uidx, const double *Uval,
                         const int32_t *orders, const int32_t *iAA2iA, int K, int nthreads,
                         const std::vector<int64_t> &partner) {
  struct Group { int64_t b0 = 0; int r = 0; std::vector<int64_t> cols; std::vector<double> vals; };
  std::vector<Group> groups;
  // row grouping
  {
    int64_t b = 0;
    while (b < nB) {
      Group g;
      g.b0 = b;
      std::vector<int64_t> cols(Uidx + Uptr[b], Uidx + Uptr[b + 1]);
      int r = 1;
      while (b + r < nB && r < UB_R) {
        bool overlap = false;
        for (int64_t q = Uptr[b + r]; q < Uptr[b + r + 1] && !overlap; ++q)
          overlap = std::find(cols.begin(), cols.end(), (int64_t)Uidx[q]) != cols.end();
        if (!overlap) break;
        cols.insert(cols.end(), Uidx + Uptr[b + r], Uidx + Uptr[b + r + 1]);
        ++r;
      }
      g.r = r;
      // representative columns (a partner pair maps to its smaller index)
      auto rep = [&](int64_t k) { return partner.empty() ? k : std::min(k, partner[k]); };
      std::vector<int64_t> reps;
      for (int64_t k : cols) reps.push_back(rep(k));
      std::sort(reps.begin(), reps.end());
      reps.erase(std::unique(reps.begin(), reps.end()), reps.end());
      g.cols = reps;
      g.vals.assign(reps.size() * UB_R, 0.0);
      for (int i = 0; i < r; ++i)
        for (int64_t q = Uptr[b + i]; q < Uptr[b + i + 1]; ++q) {
          const int64_t c = std::lower_bound(reps.begin(), reps.end(), rep(Uidx[q])) - reps.begin();
          g.vals[c * UB_R + i] += Uval[q];
        }
      if (g.cols.empty()) { g.cols.push_back(-1); g.vals.assign(UB_R, 0.0); }  // rows without nonzeros
      groups.push_back(std::move(g));
      b += r;
    }
  }
  // assignment to threads
  std::vector<size_t> order(groups.size());
  std::iota(order.begin(), order.end(), 0);
  std::stable_sort(order.begin(), order.end(), [&](size_t x, size_t y) { return groups[x].cols.size() > groups[y].cols.size(); });
  std::vector<std::vector<size_t>> own(nthreads);
  using P = std::pair<int64_t, int>;
  std::priority_queue<P, std::vector<P>, std::greater<P>> pq;
  for (int t = 0; t < nthreads; ++t) pq.push({0, t});
  URows u;
  for (size_t gi : order) {
    P top = pq.top();
    pq.pop();
    own[top.second].push_back(gi);
    top.first += (int64_t)groups[gi].cols.size();
    u.len = std::max(u.len, top.first);
    pq.push(top);
  }
  u.rec.assign((size_t)u.len * nthreads * 4, 0u);
  u.val.assign((size_t)u.len * nthreads * UB_R, 0.0);
  for (int t = 0; t < nthreads; ++t) {
    int64_t j = 0;
    for (size_t gi : own[t]) {
      const Group &g = groups[gi];
      for (size_t c = 0; c < g.cols.size(); ++c, ++j) {
        const size_t slot = (size_t)j * nthreads + t;
        uint32_t *r = &u.rec[4 * slot];
        const int64_t k = g.cols[c];
        const int ord = k < 0 ? 0 : orders[k];
        uint16_t v[6] = {0, 0, 0, 0, 0, 0};
        for (int d = 0; d < ord; ++d) v[d] = (uint16_t)iAA2iA[k * K + d];
        r[0] = v[0] | ((uint32_t)v[1] << 16);
        r[1] = v[2] | ((uint32_t)v[3] << 16);
        r[2] = v[4] | ((uint32_t)v[5] << 16);
        const bool last = (c + 1 == g.cols.size());
        r[3] = (uint32_t)g.b0 | ((uint32_t)ord << 24) | ((uint32_t)(g.r - 1) << 27) | ((last ? 1u : 0u) << 30) |
               (1u << 31);
        for (int i = 0; i < UB_R; ++i) u.val[slot * UB_R + i] = g.vals[c * UB_R + i];
      }
    }
  }
  return u;
}

}  // namespace ace
