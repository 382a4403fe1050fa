// Host symbolic analysis: pivot-group union-find, nested dissection, supernode
// borders and levels, bucket classes and the GPU panel layout with its
// deterministic gathers.
//
// The algorithm is voltax's symbolic phase (voltax/sparse.py:257-535) and
// reproduces voltax_gb300.symbolic's numpy restatement element for element:
// every tie is broken the same way (first maximum of a BFS distance, first
// lightest separator level, components labelled in order of their lowest
// vertex, stable sorts), and every floating-point comparison uses the same
// double-precision operations in the same order. Plain C++17, no
// dependencies; builds with g++ on any host.

#include "vxg_symbolic.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <mutex>
#include <new>
#include <string>
#include <system_error>
#include <thread>
#include <utility>
#include <vector>

namespace {

using i64 = int64_t;
using Vec = std::vector<i64>;

thread_local std::string g_error;

struct Error {
  int code;
  std::string msg;
};

[[noreturn]] void fail(int code, const std::string& msg) { throw Error{code, msg}; }

// Compressed rows over 0..n-1.
struct Csr {
  Vec ptr, idx;
  i64 rows() const { return (i64)ptr.size() - 1; }
  i64 begin(i64 r) const { return ptr[r]; }
  i64 end(i64 r) const { return ptr[r + 1]; }
};

// Groups `val` (one entry per source) by `key` in [0, n): sources of each key
// in ascending source order (a stable counting sort).
Csr bucket(const Vec& key, i64 n) {
  Csr c;
  c.ptr.assign(n + 1, 0);
  for (i64 k : key) c.ptr[k + 1]++;
  for (i64 i = 0; i < n; ++i) c.ptr[i + 1] += c.ptr[i];
  c.idx.resize(key.size());
  Vec fill(c.ptr.begin(), c.ptr.end() - 1);
  for (i64 s = 0; s < (i64)key.size(); ++s) c.idx[fill[key[s]]++] = s;
  return c;
}

// ---------------------------------------------------------------------------
// Pivot groups (voltax/sparse.py:257-305): union-find over the given pairs.
// union(a, b) attaches root(b) under root(a); groups are numbered by root.
// ---------------------------------------------------------------------------
Vec pivot_groups(i64 S, i64 n, const i64* ua, const i64* ub, i64* G_out) {
  Vec parent(S);
  for (i64 i = 0; i < S; ++i) parent[i] = i;
  auto find = [&](i64 a) {
    i64 root = a;
    while (parent[root] != root) root = parent[root];
    while (parent[a] != root) {
      i64 next = parent[a];
      parent[a] = root;
      a = next;
    }
    return root;
  };
  for (i64 i = 0; i < n; ++i) {
    if (ua[i] < 0 || ua[i] >= S || ub[i] < 0 || ub[i] >= S)
      fail(VXS_ERR_INVALID, "union pair outside 0..S-1");
    i64 ra = find(ua[i]), rb = find(ub[i]);
    if (ra != rb) parent[rb] = ra;
  }
  Vec root(S), rank(S, -1);
  for (i64 i = 0; i < S; ++i) {
    root[i] = find(i);
    rank[root[i]] = 0;
  }
  i64 G = 0;
  for (i64 i = 0; i < S; ++i)
    if (rank[i] == 0) rank[i] = ++G;  // roots in ascending id order
  Vec gid(S);
  for (i64 i = 0; i < S; ++i) gid[i] = rank[root[i]] - 1;
  *G_out = G;
  return gid;
}

// Runs fn(i, state) for i in [0, n) on up to VXS_THREADS threads (default:
// the hardware's, at most 8), each thread with its own default-constructed
// State; the first error is rethrown here.
template <typename State, typename Fn>
void parallel_for(i64 n, Fn&& fn) {
  i64 want = (i64)std::thread::hardware_concurrency();
  if (want <= 0) want = 1;
  want = std::min<i64>(want, 8);
  if (const char* env = std::getenv("VXS_THREADS")) {
    const long v = std::strtol(env, nullptr, 10);
    if (v > 0) want = v;
  }
  const i64 nthreads = std::max<i64>(1, std::min(want, n));
  std::atomic<i64> next{0};
  std::atomic<bool> failed{false};
  std::mutex mu;
  int code = VXS_OK;
  std::string msg;
  auto worker = [&] {
    State st;
    for (;;) {
      const i64 i = next.fetch_add(1);
      if (i >= n || failed.load()) return;
      try {
        fn(i, st);
      } catch (const Error& e) {
        std::lock_guard<std::mutex> g(mu);
        if (!failed.exchange(true)) code = e.code, msg = e.msg;
      } catch (const std::bad_alloc&) {
        std::lock_guard<std::mutex> g(mu);
        if (!failed.exchange(true)) code = VXS_ERR_NOMEM, msg = "out of host memory";
      }
    }
  };
  std::vector<std::thread> pool;
  for (i64 t = 1; t < nthreads; ++t) {
    try {
      pool.emplace_back(worker);
    } catch (const std::system_error&) {
      break;  // fewer threads: the calling thread takes the remaining items
    }
  }
  worker();
  for (std::thread& t : pool) t.join();
  if (failed.load()) fail(code, msg);
}

// ---------------------------------------------------------------------------
// Nested dissection of the group graph (voltax/sparse.py:308-378).
// ---------------------------------------------------------------------------
struct Dissection {
  const Csr& adj;
  const Vec& w;
  i64 leaf;
  Vec& loc;    // global vertex -> index in the current set, or -1 (shared by workers
               // on disjoint vertex sets)
  Vec dist, lab, queue;
  std::vector<std::pair<Vec, i64>> nodes;  // (vertex set, parent) in creation order

  Dissection(const Csr& a, const Vec& wt, i64 lf, Vec& lc) : adj(a), w(wt), leaf(lf), loc(lc) {}

  // BFS distances inside the current set from local vertex `start`.
  void bfs(const Vec& verts, i64 start) {
    i64 n = (i64)verts.size();
    dist.assign(n, -1);
    queue.resize(n);
    i64 head = 0, tail = 0;
    dist[start] = 0;
    queue[tail++] = start;
    while (head < tail) {
      i64 u = queue[head++];
      i64 g = verts[u];
      for (i64 e = adj.begin(g); e < adj.end(g); ++e) {
        i64 j = loc[adj.idx[e]];
        if (j >= 0 && dist[j] < 0) {
          dist[j] = dist[u] + 1;
          queue[tail++] = j;
        }
      }
    }
  }

  // Components inside the current set, labelled in order of their lowest
  // local vertex. Returns the count.
  i64 components(const Vec& verts) {
    i64 n = (i64)verts.size();
    lab.assign(n, -1);
    queue.resize(n);
    i64 ncomp = 0;
    for (i64 s = 0; s < n; ++s) {
      if (lab[s] >= 0) continue;
      i64 head = 0, tail = 0;
      lab[s] = ncomp;
      queue[tail++] = s;
      while (head < tail) {
        i64 u = queue[head++];
        i64 g = verts[u];
        for (i64 e = adj.begin(g); e < adj.end(g); ++e) {
          i64 j = loc[adj.idx[e]];
          if (j >= 0 && lab[j] < 0) {
            lab[j] = ncomp;
            queue[tail++] = j;
          }
        }
      }
      ++ncomp;
    }
    return ncomp;
  }

  // Dissects `first` (parent `par`) and every set it splits into, depth
  // first from one stack, appending (set, parent) to `nodes`; parents of
  // the sets created here are indices into `nodes`.
  void dissect(Vec first, i64 par0) {
    std::vector<std::pair<Vec, i64>> stack;
    stack.emplace_back(std::move(first), par0);
    while (!stack.empty()) {
      Vec verts = std::move(stack.back().first);
      i64 par = stack.back().second;
      stack.pop_back();
      i64 n = (i64)verts.size();
      if (n == 0) continue;
      for (i64 i = 0; i < n; ++i) loc[verts[i]] = i;
      auto release = [&] {
        for (i64 v : verts) loc[v] = -1;
      };
      i64 ncomp = components(verts);
      if (ncomp > 1) {
        std::vector<Vec> parts(ncomp);
        for (i64 i = 0; i < n; ++i) parts[lab[i]].push_back(verts[i]);
        release();
        for (i64 c = 0; c < ncomp; ++c) stack.emplace_back(std::move(parts[c]), par);
        continue;
      }
      i64 weight = 0;
      for (i64 v : verts) weight += w[v];
      if (weight <= leaf) {
        release();
        nodes.emplace_back(std::move(verts), par);
        continue;
      }
      // pseudo-peripheral start: up to four sweeps to the first farthest vertex
      i64 start = 0;
      for (int sweep = 0; sweep < 4; ++sweep) {
        bfs(verts, start);
        i64 far = 0;
        for (i64 i = 1; i < n; ++i)
          if (dist[i] > dist[far]) far = i;
        if (dist[far] <= dist[start] || far == start) break;
        start = far;
      }
      bfs(verts, start);
      i64 depth = *std::max_element(dist.begin(), dist.end());
      if (depth < 2) {
        release();
        nodes.emplace_back(std::move(verts), par);
        continue;
      }
      // level weights and their running sums (integers, exact in double)
      std::vector<double> lw(depth + 1, 0.0), cum(depth + 1);
      for (i64 i = 0; i < n; ++i) lw[dist[i]] += (double)w[verts[i]];
      double run = 0.0;
      for (i64 l = 0; l <= depth; ++l) cum[l] = (run += lw[l]);
      double total = cum[depth];
      i64 lv = -1;
      for (i64 l = 1; l < depth; ++l) {
        if (cum[l - 1] >= total / 3 && total - cum[l] >= total / 3) {
          if (lv < 0 || lw[l] < lw[lv]) lv = l;  // first lightest
        }
      }
      if (lv < 0) {
        i64 mid = std::lower_bound(cum.begin(), cum.end(), total / 2) - cum.begin();
        lv = std::min(std::max(mid, (i64)1), depth - 1);
      }
      Vec sep, low, high;
      for (i64 i = 0; i < n; ++i) {
        i64 d = dist[i];
        if (d > lv) {
          high.push_back(verts[i]);
        } else if (d < lv) {
          low.push_back(verts[i]);
        } else {
          bool touches = false;
          i64 g = verts[i];
          for (i64 e = adj.begin(g); e < adj.end(g) && !touches; ++e) {
            i64 j = loc[adj.idx[e]];
            touches = j >= 0 && dist[j] == lv + 1;
          }
          (touches ? sep : low).push_back(g);
        }
      }
      release();
      i64 me = (i64)nodes.size();
      nodes.emplace_back(std::move(sep), par);
      stack.emplace_back(std::move(low), me);
      stack.emplace_back(std::move(high), me);
    }
  }

  // The high-degree groups (`last`) form the root set; the rest is
  // dissected. Its connected components (the segments of a batch of
  // independent circuits) are independent subtrees: they are dissected on
  // the thread pool and appended in the order one stack visits them (the
  // last component first), so the result is that of the sequential run.
  void run(const std::vector<char>& last) {
    i64 G = adj.rows();
    i64 top = -1;
    Vec lastv, rest;
    for (i64 g = 0; g < G; ++g) (last[g] ? lastv : rest).push_back(g);
    if (!lastv.empty()) {
      nodes.emplace_back(std::move(lastv), -1);
      top = 0;
    }
    const i64 n = (i64)rest.size();
    if (n == 0) return;
    for (i64 i = 0; i < n; ++i) loc[rest[i]] = i;
    const i64 ncomp = components(rest);
    if (ncomp <= 1) {
      for (i64 v : rest) loc[v] = -1;
      dissect(std::move(rest), top);
      return;
    }
    std::vector<Vec> parts(ncomp);
    for (i64 i = 0; i < n; ++i) parts[lab[i]].push_back(rest[i]);
    for (i64 v : rest) loc[v] = -1;
    constexpr i64 kRoot = -2;  // "the parent of this component" while apart
    std::vector<std::vector<std::pair<Vec, i64>>> sub(ncomp);
    parallel_for<std::unique_ptr<Dissection>>(
        ncomp, [&](i64 c, std::unique_ptr<Dissection>& wk) {
          if (!wk) wk.reset(new Dissection(adj, w, leaf, loc));
          wk->nodes.clear();
          wk->dissect(std::move(parts[(size_t)c]), kRoot);
          sub[(size_t)c] = std::move(wk->nodes);
        });
    for (i64 c = ncomp - 1; c >= 0; --c) {
      const i64 off = (i64)nodes.size();
      for (auto& [set, p] : sub[(size_t)c]) nodes.emplace_back(std::move(set), p == kRoot ? top : p + off);
    }
  }

  // Postorder renumbering: sets and parents in elimination order.
  void postorder(std::vector<Vec>& sets, Vec& parents) {
    i64 m = (i64)nodes.size();
    Vec par(m);
    for (i64 i = 0; i < m; ++i) par[i] = nodes[i].second;
    Vec roots;
    Vec kids_key;
    for (i64 i = 0; i < m; ++i)
      if (par[i] < 0) roots.push_back(i);
    Vec owner(m);
    for (i64 i = 0; i < m; ++i) owner[i] = par[i] < 0 ? m : par[i];
    Csr kids = bucket(owner, m + 1);  // children of i in creation order
    Vec order;
    order.reserve(m);
    std::vector<std::pair<i64, bool>> todo;
    for (auto it = roots.rbegin(); it != roots.rend(); ++it) todo.emplace_back(*it, false);
    while (!todo.empty()) {
      auto [i, done] = todo.back();
      todo.pop_back();
      if (done) {
        order.push_back(i);
      } else {
        todo.emplace_back(i, true);
        for (i64 e = kids.end(i) - 1; e >= kids.begin(i); --e) todo.emplace_back(kids.idx[e], false);
      }
    }
    Vec renum(m);
    for (i64 i = 0; i < m; ++i) renum[order[i]] = i;
    sets.resize(m);
    parents.resize(m);
    for (i64 i = 0; i < m; ++i) {
      sets[i] = std::move(nodes[order[i]].first);
      i64 p = nodes[order[i]].second;
      parents[i] = p >= 0 ? renum[p] : -1;
    }
  }
};

// ---------------------------------------------------------------------------
// The plan.
// ---------------------------------------------------------------------------
// One elimination level's launch tables (ends are local CSR ends), and
// where its Schur and border sources start in the concatenated ST_SRC and
// BT_SRC.
struct LevelOut {
  Vec sn, schur_off, bord_off, st_tgt, st_end, st_src, bt_tgt, bt_end, bt_src;
  i64 schur_len = 0, bord_len = 0;
  i64 st_base = 0, bt_base = 0;
};

// The plan's fields. The per-level launch tables (LV_SN, LV_SCHUR_OFF,
// LV_BORD_OFF and the ST_* / BT_* gathers) stay in their levels' pieces
// (`lv`) and are concatenated only by the copy into the caller's array,
// level by level on the thread pool: the plan never holds a second,
// concatenated copy of its largest fields.
struct Plan {
  Vec f[VXS_N_FIELDS];
  std::vector<LevelOut> lv;
  uint32_t taken = 0;  // pieced fields already moved out (bit per field)
};

bool pieced(int field) {
  switch (field) {
    case VXS_LV_SN: case VXS_LV_SCHUR_OFF: case VXS_LV_BORD_OFF: case VXS_ST_TGT:
    case VXS_ST_PTR: case VXS_ST_SRC: case VXS_BT_TGT: case VXS_BT_PTR: case VXS_BT_SRC:
      return true;
    default:
      return false;
  }
}

// A level's piece of a pieced field (the CSR pointer fields: its local ends).
Vec& piece(LevelOut& o, int field) {
  switch (field) {
    case VXS_LV_SN: return o.sn;
    case VXS_LV_SCHUR_OFF: return o.schur_off;
    case VXS_LV_BORD_OFF: return o.bord_off;
    case VXS_ST_TGT: return o.st_tgt;
    case VXS_ST_PTR: return o.st_end;
    case VXS_ST_SRC: return o.st_src;
    case VXS_BT_TGT: return o.bt_tgt;
    case VXS_BT_PTR: return o.bt_end;
    default: return o.bt_src;
  }
}

i64 key3(i64 k, i64 r) { return k * k * k + k * k * r + k * r * r; }

// Padded cost of one bucket of `len` supernodes whose largest width and
// border are K and R (voltax/sparse.py:459-473), in the restatement's order
// of double operations.
double bucket_cost(i64 len, i64 K, i64 R) {
  if (len == 0) return 0.0;
  double a = 2.0 * (double)(K * K * K);
  double b = 2.0 * (double)K * (double)K * (double)R;
  double c = 2.0 * (double)K * (double)R * (double)R;
  return (double)len * (a + b + c + 64.0);
}

constexpr double kSplitSaving = 1e6;

struct GatherScratch {
  Vec tq;                             // target of each source, in source order
  std::vector<uint64_t> pa, pb;       // packed (target << 32 | source)
  Vec key_a, key_b, src_a, src_b;     // unpacked, when a value needs 32+ bits
};

// Unique targets of `w.tq` ascending (`tgt`), the end of each target's
// sources (`end`, CSR ends from 0) and the sources in that order, ascending
// within a target (`src`): a stable LSD radix sort of the sources by target
// (11-bit digits; sequential passes, no random access over the panel).
void gather(GatherScratch& w, i64 n_targets, Vec& tgt, Vec& end, Vec& src) {
  const i64 n = (i64)w.tq.size();
  tgt.clear();
  end.clear();
  src.clear();
  if (n == 0) return;
  constexpr int kBits = 11;
  constexpr i64 kRadix = i64(1) << kBits;
  std::vector<i64> count(kRadix);
  auto digit_passes = [&](auto&& key_of, auto&& move) {
    for (int shift = 0; shift == 0 || ((n_targets - 1) >> shift) > 0; shift += kBits) {
      std::fill(count.begin(), count.end(), 0);
      for (i64 i = 0; i < n; ++i) count[(key_of(i) >> shift) & (kRadix - 1)]++;
      i64 run = 0;
      for (i64 d = 0; d < kRadix; ++d) {
        const i64 c = count[d];
        count[d] = run;
        run += c;
      }
      for (i64 i = 0; i < n; ++i) move(i, count[(key_of(i) >> shift) & (kRadix - 1)]++);
      move(-1, 0);  // swap the buffers
    }
  };
  auto emit = [&](auto&& key_at, auto&& src_at) {
    tgt.reserve(n);
    end.reserve(n);
    src.resize(n);
    for (i64 i = 0; i < n; ++i) {
      const i64 k = key_at(i);
      if (i > 0 && k != key_at(i - 1)) end.push_back(i);
      if (i == 0 || k != key_at(i - 1)) tgt.push_back(k);
      src[i] = src_at(i);
    }
    end.push_back(n);
    tgt.shrink_to_fit();
    end.shrink_to_fit();
  };
  if (n_targets <= (i64(1) << 32) && n <= (i64(1) << 32)) {
    w.pa.resize(n);
    w.pb.resize(n);
    for (i64 s = 0; s < n; ++s) w.pa[s] = ((uint64_t)w.tq[s] << 32) | (uint64_t)s;
    digit_passes([&](i64 i) { return (i64)(w.pa[i] >> 32); },
                 [&](i64 i, i64 at) {
                   if (i < 0) w.pa.swap(w.pb);
                   else w.pb[at] = w.pa[i];
                 });
    emit([&](i64 i) { return (i64)(w.pa[i] >> 32); },
         [&](i64 i) { return (i64)(w.pa[i] & 0xffffffffu); });
  } else {
    w.key_a = w.tq;
    w.src_a.resize(n);
    for (i64 s = 0; s < n; ++s) w.src_a[s] = s;
    w.key_b.resize(n);
    w.src_b.resize(n);
    digit_passes([&](i64 i) { return w.key_a[i]; },
                 [&](i64 i, i64 at) {
                   if (i < 0) {
                     w.key_a.swap(w.key_b);
                     w.src_a.swap(w.src_b);
                   } else {
                     w.key_b[at] = w.key_a[i];
                     w.src_b[at] = w.src_a[i];
                   }
                 });
    emit([&](i64 i) { return w.key_a[i]; }, [&](i64 i) { return w.src_a[i]; });
  }
}

// Runs fn(level, scratch) for every level on up to VXS_THREADS threads.
template <typename Fn>
void run_levels(i64 nlev, Fn&& fn) {
  parallel_for<GatherScratch>(nlev, fn);
}


void build(Plan& P, i64 S, const i64* indptr, const i64* indices, i64 n_unions,
           const i64* ua, const i64* ub, i64 leaf) {
  if (S < 0 || leaf < 1) fail(VXS_ERR_INVALID, "S must be >= 0 and leaf >= 1");
  if (indptr[0] != 0) fail(VXS_ERR_INVALID, "indptr[0] must be 0");
  for (i64 i = 0; i < S; ++i)
    if (indptr[i + 1] < indptr[i]) fail(VXS_ERR_INVALID, "indptr must be non-decreasing");
  const i64 nnz = indptr[S];
  for (i64 e = 0; e < nnz; ++e)
    if (indices[e] < 0 || indices[e] >= S) fail(VXS_ERR_INVALID, "column index outside 0..S-1");

  // symmetric pattern P + P^T: row v of P, then column v of P
  Vec rows(nnz);
  for (i64 i = 0; i < S; ++i)
    for (i64 e = indptr[i]; e < indptr[i + 1]; ++e) rows[e] = i;
  Vec cols(indices, indices + nnz);
  Csr colsof = bucket(cols, S);  // entries of each column, ascending
  auto for_sym = [&](i64 v, auto&& fn) {
    for (i64 e = indptr[v]; e < indptr[v + 1]; ++e) fn(indices[e]);
    for (i64 e = colsof.begin(v); e < colsof.end(v); ++e) fn(rows[colsof.idx[e]]);
  };

  // ---- pivot groups and the group graph Q (no self loops)
  i64 G = 0;
  Vec gid = pivot_groups(S, n_unions, ua, ub, &G);
  Csr members = bucket(gid, G);  // unknowns of each group, ascending
  Vec w(G);
  for (i64 g = 0; g < G; ++g) w[g] = members.end(g) - members.begin(g);
  Csr Q;
  Q.ptr.assign(G + 1, 0);
  {
    Vec mark(G, -1);
    for (i64 g = 0; g < G; ++g) {
      for (i64 e = members.begin(g); e < members.end(g); ++e) {
        for_sym(members.idx[e], [&](i64 u) {
          i64 h = gid[u];
          if (h != g && mark[h] != g) {
            mark[h] = g;
            Q.idx.push_back(h);
          }
        });
      }
      Q.ptr[g + 1] = (i64)Q.idx.size();
    }
  }
  std::vector<char> last(G, 0);
  if (S <= 2 * leaf) {
    std::fill(last.begin(), last.end(), 1);
  } else {
    double cap = std::max(32.0, 8.0 * std::sqrt((double)G));
    for (i64 g = 0; g < G; ++g) last[g] = (double)(Q.end(g) - Q.begin(g)) > cap;
  }

  // ---- nested dissection into supernodes (group sets), postorder
  std::vector<Vec> qsets;
  Vec parents;
  {
    Vec loc(G, -1);
    Dissection nd(Q, w, leaf, loc);
    nd.run(last);
    nd.postorder(qsets, parents);
  }
  const i64 nsn = (i64)qsets.size();

  // ---- supernodes: sorted unknowns of their groups
  Vec& sn_ptr = P.f[VXS_SN_PTR];
  Vec& sn_idx = P.f[VXS_SN_IDX];
  sn_ptr.assign(nsn + 1, 0);
  sn_idx.reserve(S);
  for (i64 i = 0; i < nsn; ++i) {
    i64 at = (i64)sn_idx.size();
    for (i64 g : qsets[i])
      for (i64 e = members.begin(g); e < members.end(g); ++e) sn_idx.push_back(members.idx[e]);
    std::sort(sn_idx.begin() + at, sn_idx.end());
    sn_ptr[i + 1] = (i64)sn_idx.size();
  }
  if ((i64)sn_idx.size() != S) fail(VXS_ERR_INVALID, "supernodes do not cover the unknowns");
  Vec& sn_of = P.f[VXS_SN_OF];
  Vec& pos_in = P.f[VXS_POS_IN];
  sn_of.assign(S, -1);
  pos_in.assign(S, -1);
  for (i64 i = 0; i < nsn; ++i)
    for (i64 e = sn_ptr[i]; e < sn_ptr[i + 1]; ++e) {
      sn_of[sn_idx[e]] = i;
      pos_in[sn_idx[e]] = e - sn_ptr[i];
    }

  // ---- borders and levels
  Vec owner(nsn);
  for (i64 i = 0; i < nsn; ++i) owner[i] = parents[i] < 0 ? nsn : parents[i];
  Csr kids = bucket(owner, nsn + 1);
  Vec& bd_ptr = P.f[VXS_BD_PTR];
  Vec& bd_idx = P.f[VXS_BD_IDX];
  Vec& level = P.f[VXS_LEVEL];
  bd_ptr.assign(nsn + 1, 0);
  level.assign(nsn, 0);
  {
    Vec cand;
    for (i64 i = 0; i < nsn; ++i) {
      cand.clear();
      for (i64 e = sn_ptr[i]; e < sn_ptr[i + 1]; ++e)
        for_sym(sn_idx[e], [&](i64 u) {
          if (sn_of[u] > i) cand.push_back(u);
        });
      for (i64 e = kids.begin(i); e < kids.end(i); ++e) {
        i64 c = kids.idx[e];
        for (i64 b = bd_ptr[c]; b < bd_ptr[c + 1]; ++b)
          if (sn_of[bd_idx[b]] > i) cand.push_back(bd_idx[b]);
        level[i] = std::max(level[i], level[c] + 1);
      }
      std::sort(cand.begin(), cand.end());
      cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
      bd_idx.insert(bd_idx.end(), cand.begin(), cand.end());
      bd_ptr[i + 1] = (i64)bd_idx.size();
    }
  }
  Vec& K = P.f[VXS_K];
  Vec& R = P.f[VXS_R];
  K.resize(nsn);
  R.resize(nsn);
  for (i64 i = 0; i < nsn; ++i) {
    K[i] = sn_ptr[i + 1] - sn_ptr[i];
    R[i] = bd_ptr[i + 1] - bd_ptr[i];
  }
  i64 nlev = 0;
  for (i64 l : level) nlev = std::max(nlev, l + 1);
  Csr by_level = bucket(level, nlev);  // supernodes of each level, ascending

  // ---- bucket classes (voltax/sparse.py:459-473)
  Vec& cls_ptr = P.f[VXS_CLS_PTR];
  Vec& cls_idx = P.f[VXS_CLS_IDX];
  cls_ptr.assign(1, 0);
  for (i64 lv = 0; lv < nlev; ++lv) {
    Vec sel(by_level.idx.begin() + by_level.begin(lv), by_level.idx.begin() + by_level.end(lv));
    std::stable_sort(sel.begin(), sel.end(),
                     [&](i64 a, i64 b) { return key3(K[a], R[a]) < key3(K[b], R[b]); });
    i64 n = (i64)sel.size();
    Vec pk(n + 1, 0), pr(n + 1, 0), sk(n + 1, 0), sr(n + 1, 0);
    for (i64 c = 0; c < n; ++c) {
      pk[c + 1] = std::max(pk[c], K[sel[c]]);
      pr[c + 1] = std::max(pr[c], R[sel[c]]);
    }
    for (i64 c = n - 1; c >= 0; --c) {
      sk[c] = std::max(sk[c + 1], K[sel[c]]);
      sr[c] = std::max(sr[c + 1], R[sel[c]]);
    }
    auto pre = [&](i64 c) { return bucket_cost(c, pk[c], pr[c]); };
    auto suf = [&](i64 c) { return bucket_cost(n - c, sk[c], sr[c]); };
    i64 cut = 0;
    double best = pre(0) + suf(0);
    for (i64 c = 1; c < n; ++c) {
      double v = pre(c) + suf(c);
      if (v < best) {
        best = v;
        cut = c;
      }
    }
    if (suf(0) - pre(cut) - suf(cut) < kSplitSaving) cut = 0;
    if (cut > 0) {
      cls_idx.insert(cls_idx.end(), sel.begin(), sel.begin() + cut);
      cls_ptr.push_back((i64)cls_idx.size());
    }
    cls_idx.insert(cls_idx.end(), sel.begin() + cut, sel.end());
    cls_ptr.push_back((i64)cls_idx.size());
  }

  // ---- GPU layout: unpadded panels in supernode order
  Vec& panel = P.f[VXS_PANEL];
  panel.assign(nsn, 0);
  for (i64 i = 1; i < nsn; ++i) panel[i] = panel[i - 1] + K[i - 1] * K[i - 1] + 2 * K[i - 1] * R[i - 1];

  auto bpos = [&](i64 o, i64 v) {
    auto b0 = bd_idx.begin() + bd_ptr[o], b1 = bd_idx.begin() + bd_ptr[o + 1];
    auto it = std::lower_bound(b0, b1, v);
    if (it == b1 || *it != v) fail(VXS_ERR_STRUCTURE, "entry outside the supernodal factor structure");
    return (i64)(it - b0);
  };
  auto position = [&](i64 u, i64 v) {
    i64 su = sn_of[u], sv = sn_of[v];
    if (su == sv) return panel[su] + pos_in[u] * K[su] + pos_in[v];
    if (su < sv) return panel[su] + K[su] * K[su] + pos_in[u] * R[su] + bpos(su, v);
    return panel[sv] + K[sv] * K[sv] + K[sv] * R[sv] + bpos(sv, u) * K[sv] + pos_in[v];
  };
  Vec& a_pos = P.f[VXS_A_POS];
  a_pos.resize(nnz);
  for (i64 e = 0; e < nnz; ++e) a_pos[e] = position(rows[e], indices[e]);

  // ---- per-level launch tables with deterministic gathers. Levels are
  // independent (every input is read-only here): a small pool of threads
  // builds them, and they are concatenated in level order.
  const i64 work_len = nsn ? panel[nsn - 1] + K[nsn - 1] * K[nsn - 1] + 2 * K[nsn - 1] * R[nsn - 1] : 0;
  std::vector<LevelOut> outs(nlev);
  auto build_level = [&](i64 lv, GatherScratch& w, LevelOut& o) {
    o.sn.assign(by_level.idx.begin() + by_level.begin(lv), by_level.idx.begin() + by_level.end(lv));
    std::stable_sort(o.sn.begin(), o.sn.end(),
                     [&](i64 a, i64 b) { return key3(K[a], R[a]) > key3(K[b], R[b]); });
    i64 soff = 0, boff = 0;
    w.tq.clear();
    for (i64 j : o.sn) {
      o.schur_off.push_back(soff);
      o.bord_off.push_back(boff);
      const i64 r = R[j];
      const i64* b = bd_idx.data() + bd_ptr[j];
      for (i64 x = 0; x < r; ++x)  // row-major r x r block: source soff + x*r + y
        for (i64 y = 0; y < r; ++y) w.tq.push_back(position(b[x], b[y]));
      soff += r * r;
      boff += r;
    }
    o.schur_len = soff;
    o.bord_len = boff;
    gather(w, work_len, o.st_tgt, o.st_end, o.st_src);
    w.tq.clear();
    for (i64 j : o.sn) w.tq.insert(w.tq.end(), bd_idx.begin() + bd_ptr[j], bd_idx.begin() + bd_ptr[j + 1]);
    gather(w, S, o.bt_tgt, o.bt_end, o.bt_src);
  };
  run_levels(nlev, [&](i64 lv, GatherScratch& w) { build_level(lv, w, outs[lv]); });

  Vec& lv_ptr = P.f[VXS_LV_PTR];
  Vec& lv_schur_len = P.f[VXS_LV_SCHUR_LEN];
  Vec& lv_bord_len = P.f[VXS_LV_BORD_LEN];
  Vec& lv_st_ptr = P.f[VXS_LV_ST_PTR];
  Vec& lv_bt_ptr = P.f[VXS_LV_BT_PTR];
  lv_ptr.assign(1, 0);
  lv_st_ptr.assign(1, 0);
  lv_bt_ptr.assign(1, 0);
  i64 n_ss = 0, n_bs = 0;
  for (LevelOut& o : outs) {  // level order
    o.st_base = n_ss;
    o.bt_base = n_bs;
    n_ss += (i64)o.st_src.size();
    n_bs += (i64)o.bt_src.size();
    lv_ptr.push_back(lv_ptr.back() + (i64)o.sn.size());
    lv_schur_len.push_back(o.schur_len);
    lv_bord_len.push_back(o.bord_len);
    lv_st_ptr.push_back(lv_st_ptr.back() + (i64)o.st_tgt.size());
    lv_bt_ptr.push_back(lv_bt_ptr.back() + (i64)o.bt_tgt.size());
  }
  P.lv = std::move(outs);

  P.f[VXS_GID] = std::move(gid);
  P.f[VXS_PARENT] = std::move(parents);
}

}  // namespace

struct vxs_plan {
  Plan p;
};

extern "C" {

int vxs_plan_create(int64_t S, const int64_t* indptr, const int64_t* indices,
                    int64_t n_unions, const int64_t* union_a, const int64_t* union_b,
                    int64_t leaf, vxs_plan** out) {
  if (!out || !indptr || (S > 0 && !indices && indptr[S] > 0) || n_unions < 0 ||
      (n_unions > 0 && (!union_a || !union_b))) {
    g_error = "null pointer or negative count";
    return VXS_ERR_INVALID;
  }
  *out = nullptr;
  vxs_plan* p = nullptr;
  try {
    p = new vxs_plan;
    build(p->p, S, indptr, indices, n_unions, union_a, union_b, leaf);
  } catch (const Error& e) {
    delete p;
    g_error = e.msg;
    return e.code;
  } catch (const std::bad_alloc&) {
    delete p;
    g_error = "out of host memory";
    return VXS_ERR_NOMEM;
  }
  *out = p;
  return VXS_OK;
}

int64_t vxs_plan_len(const vxs_plan* p, int32_t field) {
  if (!p || field < 0 || field >= VXS_N_FIELDS) return -1;
  if (!pieced(field)) return (int64_t)p->p.f[field].size();
  if ((p->p.taken >> field) & 1u) return 0;
  int64_t n = (field == VXS_ST_PTR || field == VXS_BT_PTR) ? 1 : 0;
  for (const LevelOut& o : p->p.lv) n += (int64_t)piece(const_cast<LevelOut&>(o), field).size();
  return n;
}

int vxs_plan_copy(const vxs_plan* p, int32_t field, int64_t* dst) {
  if (!p || field < 0 || field >= VXS_N_FIELDS) {
    g_error = "unknown plan field";
    return VXS_ERR_INVALID;
  }
  if (vxs_plan_len(p, field) > 0 && !dst) {
    g_error = "null destination";
    return VXS_ERR_INVALID;
  }
  if (!pieced(field)) {
    const Vec& v = p->p.f[field];
    if (!v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(int64_t));
    return VXS_OK;
  }
  if ((p->p.taken >> field) & 1u) return VXS_OK;  // already moved out: nothing left
  // each level's piece at its offset; a pointer field's local ends shifted
  // by where the level's sources start
  const bool ends = field == VXS_ST_PTR || field == VXS_BT_PTR;
  std::vector<LevelOut>& lv = const_cast<std::vector<LevelOut>&>(p->p.lv);
  const i64 nlev = (i64)lv.size();
  Vec off(nlev + 1, ends ? 1 : 0);
  for (i64 L = 0; L < nlev; ++L) off[L + 1] = off[L] + (i64)piece(lv[L], field).size();
  if (ends) dst[0] = 0;
  try {
    parallel_for<char>(nlev, [&](i64 L, char&) {
      const Vec& v = piece(lv[L], field);
      int64_t* out = dst + off[L];
      if (ends) {
        const i64 base = field == VXS_ST_PTR ? lv[L].st_base : lv[L].bt_base;
        for (size_t i = 0; i < v.size(); ++i) out[i] = base + v[i];
      } else if (!v.empty()) {
        std::memcpy(out, v.data(), v.size() * sizeof(int64_t));
      }
    });
  } catch (const Error& e) {
    g_error = e.msg;
    return e.code;
  }
  return VXS_OK;
}

int vxs_plan_take(vxs_plan* p, int32_t field, int64_t* dst) {
  const int rc = vxs_plan_copy(p, field, dst);
  if (rc == VXS_OK) {
    if (pieced(field)) {
      for (LevelOut& o : p->p.lv) Vec().swap(piece(o, field));
      p->p.taken |= 1u << field;
    } else
      Vec().swap(p->p.f[field]);
  }
  return rc;
}

void vxs_plan_destroy(vxs_plan* p) { delete p; }

const char* vxs_last_error(void) { return g_error.c_str(); }

}  // extern "C"
