#include "bvh_build.h"
#include "../kernels/bvh_device.h"
#include "runtime.h"

#include <math.h>
#include <string.h>

#include <algorithm>
#include <array>
#include <atomic>
#include <cfloat>
#include <thread>
#include <stdlib.h>

namespace illume {

static thread_local int t_thread_share = 0;   // 0: no share set on this thread

static int all_build_threads() {
  const char* e = getenv("ILLUME_BUILD_THREADS");
  if (e && atoi(e) > 0) return std::min(256, atoi(e));
  return std::max(1, std::min(16, (int)std::thread::hardware_concurrency()));
}

int build_threads() { return t_thread_share > 0 ? t_thread_share : all_build_threads(); }

BuildThreadShare::BuildThreadShare(int share) : saved_(t_thread_share) { t_thread_share = std::max(1, share); }
BuildThreadShare::~BuildThreadShare() { t_thread_share = saved_; }

int build_thread_share(const int* sizes, int count, int builders) {
  constexpr int kLarge = 1 << 15;   // meshes below this build on one thread anyway
  int large = 0;
  for (int i = 0; i < count; ++i) large += sizes[i] >= kLarge;
  const int all = build_threads();
  if (large <= 1) return all;
  return std::max(1, all / std::max(1, std::min(large, builders)));
}

namespace {

// fn(t, begin, end) on contiguous chunks of [0, n), chunk t on thread t (the caller runs
// chunk 0), with at most build_threads() chunks of at least min_chunk items each. Every
// use combines the chunks' results in chunk order or by min / max / integer sums, so the
// result does not depend on the number of threads.
template <class Fn>
void parallel_chunks(size_t n, size_t min_chunk, Fn&& fn) {
  const size_t want = std::max<size_t>(1, n / std::max<size_t>(1, min_chunk));
  const int threads = (int)std::min<size_t>((size_t)build_threads(), want);
  if (threads <= 1) {
    fn(0, (size_t)0, n);
    return;
  }
  const size_t step = (n + threads - 1) / threads;
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) {
    const size_t b = std::min(n, t * step), e = std::min(n, b + step);
    pool.emplace_back([&fn, t, b, e] { fn(t, b, e); });
  }
  fn(0, (size_t)0, std::min(n, step));
  for (auto& th : pool) th.join();
}

struct Box {
  double lo[3], hi[3];
  void reset() {
    for (int a = 0; a < 3; ++a) { lo[a] = INFINITY; hi[a] = -INFINITY; }
  }
  void grow(const Box& b) {
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], b.lo[a]); hi[a] = std::max(hi[a], b.hi[a]); }
  }
  void grow_pt(const double* p) {
    for (int a = 0; a < 3; ++a) { lo[a] = std::min(lo[a], p[a]); hi[a] = std::max(hi[a], p[a]); }
  }
  double area() const {
    const double dx = hi[0] - lo[0], dy = hi[1] - lo[1], dz = hi[2] - lo[2];
    if (dx < 0 || dy < 0 || dz < 0) return 0.0;
    return 2.0 * (dx * dy + dy * dz + dz * dx);
  }
};

struct BNode {
  Box box;
  int left = -1, right = -1;  // children (binary tree), -1 for leaves
  int first = 0, count = 0;   // leaf range in the prim order
};

float down(double d) {
  float f = (float)d;
  if ((double)f > d) f = nextafterf(f, -INFINITY);
  return f;
}
float up(double d) {
  float f = (float)d;
  if ((double)f < d) f = nextafterf(f, INFINITY);
  return f;
}

struct Work { int node, first, count; };

// The split of node w in the top-down binned SAH build (16 bins per axis on centroids):
// nd gets the node's box and range; returns the first position of the right child in
// `order` (the range partitioned), or -1 when the node is a leaf. With threads_free, the
// bounds and the bins of a large node are gathered on the host threads (minima, maxima
// and counts: the same values on any number of threads); the partition is sequential.
int split_node(const Work& w, const std::vector<Box>& boxes, const std::vector<double>& ctr, std::vector<int>& order,
               int max_leaf, bool threads_free, BNode& nd) {
  constexpr int kBins = 16;
  constexpr int kParallelNode = 1 << 16;   // nodes of at least this many primitives
  constexpr size_t kChunk = 1 << 14;
  const bool par = threads_free && w.count >= kParallelNode;
  auto over = [&](auto&& body) {   // body(part, begin, end) over the node's range
    if (par) parallel_chunks((size_t)w.count, kChunk, body);
    else body(0, (size_t)0, (size_t)w.count);
  };
  const int nparts = par ? build_threads() : 1;
  nd = BNode();
  nd.box.reset();
  Box cb;
  cb.reset();
  {
    std::array<Box, 2> one;   // small nodes: no heap work per node
    std::vector<std::array<Box, 2>> many(par ? nparts : 0);
    std::array<Box, 2>* part = par ? many.data() : &one;
    for (int t = 0; t < nparts; ++t) { part[t][0].reset(); part[t][1].reset(); }
    over([&](int t, size_t b, size_t e) {
      Box bx = part[t][0], cx = part[t][1];
      for (size_t i = b; i < e; ++i) {
        const int p = order[w.first + i];
        bx.grow(boxes[p]);
        cx.grow_pt(&ctr[3 * (size_t)p]);
      }
      part[t][0] = bx;
      part[t][1] = cx;
    });
    for (int t = 0; t < nparts; ++t) { nd.box.grow(part[t][0]); cb.grow(part[t][1]); }
  }
  nd.first = w.first;
  nd.count = w.count;
  const double parent_area = nd.box.area();
  const double leaf_cost = (double)w.count;
  double best_cost = INFINITY;
  int best_axis = -1, best_bin = -1;
  if (w.count > 1) {
    // the bins of the three axes in one sweep over the node's primitives
    bool live[3];
    double k[3];
    for (int a = 0; a < 3; ++a) {
      const double ext = cb.hi[a] - cb.lo[a];
      live[a] = ext > 0;
      k[a] = live[a] ? kBins / ext : 0.0;
    }
    struct Bins { Box bb[3][kBins]; int bc[3][kBins]; };
    Bins one;
    std::vector<Bins> many(par ? nparts : 0);
    Bins* part = par ? many.data() : &one;
    for (int t = 0; t < nparts; ++t)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < kBins; ++b) { part[t].bb[a][b].reset(); part[t].bc[a][b] = 0; }
    over([&](int t, size_t b0, size_t e0) {
      Bins& q = part[t];
      for (size_t i = b0; i < e0; ++i) {
        const int p = order[w.first + i];
        for (int a = 0; a < 3; ++a) {
          if (!live[a]) continue;
          int b = (int)((ctr[3 * (size_t)p + a] - cb.lo[a]) * k[a]);
          b = std::min(std::max(b, 0), kBins - 1);
          q.bb[a][b].grow(boxes[p]);
          q.bc[a][b]++;
        }
      }
    });
    for (int t = 1; t < nparts; ++t)
      for (int a = 0; a < 3; ++a)
        for (int b = 0; b < kBins; ++b) {
          part[0].bb[a][b].grow(part[t].bb[a][b]);
          part[0].bc[a][b] += part[t].bc[a][b];
        }
    for (int a = 0; a < 3; ++a) {
      if (!live[a]) continue;
      const Box* bb = part[0].bb[a];
      const int* bc = part[0].bc[a];
      double rarea[kBins];
      int rcount[kBins];
      Box acc;
      acc.reset();
      int cnt = 0;
      for (int b = kBins - 1; b > 0; --b) {
        acc.grow(bb[b]);
        cnt += bc[b];
        rarea[b] = acc.area();
        rcount[b] = cnt;
      }
      acc.reset();
      cnt = 0;
      for (int b = 0; b < kBins - 1; ++b) {
        acc.grow(bb[b]);
        cnt += bc[b];
        if (cnt == 0 || rcount[b + 1] == 0) continue;
        const double cost = 1.0 + (acc.area() * cnt + rarea[b + 1] * rcount[b + 1]) / std::max(parent_area, 1e-300);
        if (cost < best_cost) { best_cost = cost; best_axis = a; best_bin = b; }
      }
    }
  }
  const bool make_leaf = w.count == 1 || (w.count <= max_leaf && leaf_cost <= best_cost);
  if (make_leaf) return -1;
  int mid;
  if (best_axis < 0) {
    // all centroids coincide (or no valid split): object median
    mid = w.first + w.count / 2;
  } else {
    const double ext = cb.hi[best_axis] - cb.lo[best_axis];
    const double k = kBins / ext;
    auto it = std::partition(order.begin() + w.first, order.begin() + w.first + w.count, [&](int p) {
      int b = (int)((ctr[3 * (size_t)p + best_axis] - cb.lo[best_axis]) * k);
      b = std::min(std::max(b, 0), kBins - 1);
      return b <= best_bin;
    });
    mid = (int)(it - order.begin());
    if (mid == w.first || mid == w.first + w.count) mid = w.first + w.count / 2;
  }
  return mid;
}

// One step of a sequential build: the node of `w` becomes a leaf, or is split and its two
// children are pushed.
void build_step(const Work& w, const std::vector<Box>& boxes, const std::vector<double>& ctr, std::vector<int>& order,
                int max_leaf, std::vector<BNode>& nodes, std::vector<Work>& stack) {
  BNode nd;
  const int mid = split_node(w, boxes, ctr, order, max_leaf, false, nd);
  if (mid < 0) {
    nodes[w.node] = nd;
    return;
  }
  nd.left = (int)nodes.size();
  nd.right = nd.left + 1;
  nodes.emplace_back();
  nodes.emplace_back();
  nodes[w.node] = nd;
  stack.push_back({nd.right, mid, w.first + w.count - mid});
  stack.push_back({nd.left, w.first, mid - w.first});
}

// Collapse of a binary tree into nodes of up to K children that minimises the summed box
// area of the K-wide nodes (the surface-area cost of their visits; the leaves are the
// binary tree's either way). F[x][j - 1] = the least area of the K-wide nodes below
// binary node x when x may fill up to j child slots of its parent: x itself as a node (its
// area plus the best split of its K slots between its children, split[x]), or x opened and
// its slots split between its children (choice[x][j - 1] = the left child's share).
// Leaves cost nothing and fill one slot. Ties keep the lower split.
template <int K>
struct WideCollapse {
  const std::vector<BNode>& bn;
  std::vector<std::array<double, K>> F;
  std::vector<std::array<int8_t, K>> choice;
  std::vector<int8_t> split;

  explicit WideCollapse(const std::vector<BNode>& b) : bn(b), F(b.size()), choice(b.size()), split(b.size(), 0) {
    // children before their parents: both builders number a node's children after the
    // node, so a sweep by descending index is bottom-up (a post-order walk otherwise)
    const int n = (int)bn.size();
    bool ordered = true;
    for (int x = 0; x < n && ordered; ++x) ordered = bn[x].left < 0 || (bn[x].left > x && bn[x].right > x);
    std::vector<int> post;
    if (!ordered) {
      post.reserve(bn.size());
      std::vector<std::pair<int, bool>> st{{0, false}};
      while (!st.empty()) {
        const auto [x, seen] = st.back();
        st.pop_back();
        if (seen || bn[x].left < 0) { post.push_back(x); continue; }
        st.push_back({x, true});
        st.push_back({bn[x].right, false});
        st.push_back({bn[x].left, false});
      }
    }
    for (int q = 0; q < n; ++q) {
      const int x = ordered ? n - 1 - q : post[q];
      if (bn[x].left < 0) {
        F[x].fill(0.0);
        choice[x].fill(0);
        continue;
      }
      const int L = bn[x].left, R = bn[x].right;
      double g = INFINITY;
      for (int m = 1; m < K; ++m) {
        const double c = F[L][m - 1] + F[R][K - m - 1];
        if (c < g) { g = c; split[x] = (int8_t)m; }
      }
      F[x][0] = bn[x].box.area() + g;
      choice[x][0] = 0;
      for (int j = 2; j <= K; ++j) {
        double best = F[x][0];
        int8_t ch = 0;
        for (int m = 1; m < j; ++m) {
          const double c = F[L][m - 1] + F[R][j - m - 1];
          if (c < best) { best = c; ch = (int8_t)m; }
        }
        F[x][j - 1] = best;
        choice[x][j - 1] = ch;
      }
    }
  }

  // The children of the K-wide node made from inner binary node x (binary nodes, left
  // to right), into out[0..K); returns their count.
  int children(int x, int* out) const {
    int nc = 0;
    // at most K pending entries: each holds at least one of the node's K slots
    int wy[2 * K], wj[2 * K], sp = 0;
    wy[sp] = bn[x].right; wj[sp++] = K - split[x];
    wy[sp] = bn[x].left; wj[sp++] = split[x];
    while (sp > 0) {
      --sp;
      const int y = wy[sp], j = wj[sp];
      if (bn[y].left < 0 || choice[y][j - 1] == 0) { out[nc++] = y; continue; }
      const int m = choice[y][j - 1];
      wy[sp] = bn[y].right; wj[sp++] = j - m;
      wy[sp] = bn[y].left; wj[sp++] = m;
    }
    return nc;
  }
};

// Binned SAH build; returns nodes (root at 0) and fills order. The top of the tree is
// split level by level until the pending subtrees are small; those are built on the host
// cores (each into its own node list, on a disjoint range of `order`) and stitched in
// the order a depth-first build sets them aside. Neither the splits nor the size at which
// subtrees are set aside depend on the thread count, so the node arrays are identical on
// any number of cores.
std::vector<BNode> build_binary(const std::vector<Box>& boxes, std::vector<int>& order, int max_leaf) {
  const int N = (int)boxes.size();
  order.resize(N);
  for (int i = 0; i < N; ++i) order[i] = i;
  std::vector<double> ctr((size_t)N * 3);
  parallel_chunks((size_t)N, 1 << 15, [&](int, size_t b, size_t e) {
    for (size_t i = b; i < e; ++i)
      for (int a = 0; a < 3; ++a) ctr[3 * i + a] = 0.5 * (boxes[i].lo[a] + boxes[i].hi[a]);
  });
  std::vector<BNode> nodes;
  nodes.reserve(2 * (size_t)N + 1);
  nodes.emplace_back();
  const int threads = build_threads();
  const int grain = N > 20000 ? std::max(4096, N / 128) : N + 1;
  std::vector<Work> deferred;
  {
    // The top of the tree, level by level: each node of a level is split on its own
    // range of `order` (a level of many nodes on the threads node by node, one of few
    // nodes with each node's bins gathered on all threads); nodes of at most `grain`
    // primitives (and more than a leaf's) are set aside for the subtree builds. A
    // depth-first replay then numbers the nodes and lists the set-aside subtrees as a
    // sequential depth-first build would: the arrays do not depend on the threads.
    struct Top {
      Work w;
      BNode nd;
      int kid = -1;            // left child in `top` (the right one is kid + 1); -1: a leaf
      bool deferred = false;
    };
    std::vector<Top> top(1);
    top[0].w = Work{0, 0, N};
    std::vector<int> level{0}, todo, mids, next_level;
    while (!level.empty()) {
      todo.clear();
      for (int id : level) {
        const Work& w = top[id].w;
        if (w.count <= grain && w.count > max_leaf) top[id].deferred = true;
        else todo.push_back(id);
      }
      mids.assign(todo.size(), -1);
      if ((int)todo.size() < threads) {
        for (size_t q = 0; q < todo.size(); ++q)
          mids[q] = split_node(top[todo[q]].w, boxes, ctr, order, max_leaf, true, top[todo[q]].nd);
      } else {
        std::atomic<size_t> nx{0};
        auto lw = [&]() {
          for (size_t q = nx++; q < todo.size(); q = nx++)
            mids[q] = split_node(top[todo[q]].w, boxes, ctr, order, max_leaf, false, top[todo[q]].nd);
        };
        std::vector<std::thread> lp;
        for (int t = 1; t < threads; ++t) lp.emplace_back(lw);
        lw();
        for (auto& th : lp) th.join();
      }
      next_level.clear();
      for (size_t q = 0; q < todo.size(); ++q) {
        if (mids[q] < 0) continue;
        const Work w = top[todo[q]].w;
        const int kid = (int)top.size();
        top[todo[q]].kid = kid;
        top.emplace_back();
        top.back().w = Work{-1, w.first, mids[q] - w.first};
        top.emplace_back();
        top.back().w = Work{-1, mids[q], w.first + w.count - mids[q]};
        next_level.push_back(kid);
        next_level.push_back(kid + 1);
      }
      level.swap(next_level);
    }
    std::vector<std::pair<int, int>> st{{0, 0}};   // (node of `top`, its slot in `nodes`)
    while (!st.empty()) {
      const auto [id, slot] = st.back();
      st.pop_back();
      const Top& t = top[id];
      if (t.deferred) { deferred.push_back(Work{slot, t.w.first, t.w.count}); continue; }
      BNode nd = t.nd;
      if (t.kid < 0) { nodes[slot] = nd; continue; }
      nd.left = (int)nodes.size();
      nd.right = nd.left + 1;
      nodes.emplace_back();
      nodes.emplace_back();
      nodes[slot] = nd;
      st.push_back({t.kid + 1, nd.right});
      st.push_back({t.kid, nd.left});
    }
  }
  if (deferred.empty()) return nodes;
  std::vector<std::vector<BNode>> sub(deferred.size());
  std::atomic<size_t> next{0};
  auto worker = [&]() {
    for (size_t k = next++; k < deferred.size(); k = next++) {
      std::vector<BNode>& sn = sub[k];
      sn.reserve(2 * (size_t)deferred[k].count + 1);
      sn.emplace_back();
      std::vector<Work> st{{0, deferred[k].first, deferred[k].count}};
      while (!st.empty()) {
        const Work w = st.back();
        st.pop_back();
        build_step(w, boxes, ctr, order, max_leaf, sn, st);
      }
    }
  };
  std::vector<std::thread> pool;
  for (int t = 1; t < threads; ++t) pool.emplace_back(worker);
  worker();
  for (auto& th : pool) th.join();
  // stitch: a subtree's root replaces its placeholder, the rest is appended in the
  // order the subtrees were set aside (subtree k's index j >= 1 -> base[k] + j)
  std::vector<size_t> base(deferred.size());
  size_t total = nodes.size();
  for (size_t k = 0; k < deferred.size(); ++k) {
    base[k] = total - 1;
    total += sub[k].size() - 1;
  }
  nodes.resize(total);
  std::atomic<size_t> nk{0};
  auto stitch = [&]() {
    for (size_t k = nk++; k < deferred.size(); k = nk++) {
      const std::vector<BNode>& sn = sub[k];
      const int b = (int)base[k];
      auto remap = [&](BNode n) {
        if (n.left >= 0) { n.left += b; n.right += b; }
        return n;
      };
      nodes[deferred[k].node] = remap(sn[0]);
      for (size_t j = 1; j < sn.size(); ++j) nodes[base[k] + j] = remap(sn[j]);
    }
  };
  std::vector<std::thread> sp;
  for (int t = 1; t < threads; ++t) sp.emplace_back(stitch);
  stitch();
  for (auto& th : sp) th.join();
  return nodes;
}

// A triangle record: three vertices, the primitive index in the first one's w.
void put_tri(float4* out, const float* P, const int* tri, int prim) {
  const float* a = P + 3 * (size_t)tri[0];
  const float* b = P + 3 * (size_t)tri[1];
  const float* c = P + 3 * (size_t)tri[2];
  float w;
  memcpy(&w, &prim, 4);
  out[0] = float4{a[0], a[1], a[2], w};
  out[1] = float4{b[0], b[1], b[2], 0.0f};
  out[2] = float4{c[0], c[1], c[2], 0.0f};
}
void put_tri(std::vector<float4>& out, const float* P, const int* tri, int prim) {
  out.resize(out.size() + 3);
  put_tri(&out[out.size() - 3], P, tri, prim);
}

int tree_depth(const std::vector<BNode>& n, int root) {
  int best = 0;
  std::vector<std::pair<int, int>> st{{root, 1}};
  while (!st.empty()) {
    const auto [i, d] = st.back();
    st.pop_back();
    if (n[i].left < 0) { best = std::max(best, d); continue; }
    st.push_back({n[i].right, d + 1});
    st.push_back({n[i].left, d + 1});
  }
  return best;
}

}  // namespace

namespace {

// The host tree of a device cluster tree: leaves of up to max_leaf primitives where the
// surface-area cost says a leaf is cheaper than the subtree below it (cost of a leaf =
// its primitives, of an inner node = 1 + the children's costs weighted by their share of
// its box area, the same units as build_step), nodes and `order` in depth-first order
// (root at 0, left subtree first). Cluster nodes are numbered after their children, so
// one ascending sweep is bottom-up.
std::vector<BNode> tree_from_clusters(const ClusterTree& ct, int max_leaf, std::vector<int>& order) {
  const int n = ct.n, total = 2 * n - 1;
  std::vector<int> cnt(total);
  std::vector<char> leaf(total);
  std::vector<double> cost(total), area(total);
  auto box_of = [&](int id) {
    Box b;
    for (int a = 0; a < 3; ++a) {
      b.lo[a] = ct.box[6 * (size_t)id + a];
      b.hi[a] = ct.box[6 * (size_t)id + 3 + a];
    }
    return b;
  };
  for (int id = 0; id < total; ++id) {
    area[id] = box_of(id).area();
    if (id < n) {
      cnt[id] = 1;
      cost[id] = 1.0;
      leaf[id] = 1;
      continue;
    }
    const int l = ct.child[2 * (size_t)(id - n)], r = ct.child[2 * (size_t)(id - n) + 1];
    cnt[id] = cnt[l] + cnt[r];
    const double split = 1.0 + (area[l] * cost[l] + area[r] * cost[r]) / std::max(area[id], 1e-300);
    leaf[id] = cnt[id] <= max_leaf && (double)cnt[id] <= split;
    cost[id] = leaf[id] ? (double)cnt[id] : split;
  }
  std::vector<BNode> nodes;
  nodes.reserve(2 * (size_t)n);
  order.clear();
  order.reserve(n);
  nodes.emplace_back();
  std::vector<std::pair<int, int>> st{{ct.root, 0}};
  std::vector<int> sub;
  while (!st.empty()) {
    const int id = st.back().first, bi = st.back().second;
    st.pop_back();
    nodes[bi].box = box_of(id);
    if (leaf[id]) {
      nodes[bi].first = (int)order.size();
      nodes[bi].count = cnt[id];
      sub.assign(1, id);
      while (!sub.empty()) {   // the leaf's primitives, left to right
        const int k = sub.back();
        sub.pop_back();
        if (k < n) {
          order.push_back(ct.prim[k]);
        } else {
          sub.push_back(ct.child[2 * (size_t)(k - n) + 1]);
          sub.push_back(ct.child[2 * (size_t)(k - n)]);
        }
      }
    } else {
      const int l = (int)nodes.size();
      nodes.emplace_back();
      nodes.emplace_back();
      nodes[bi].left = l;
      nodes[bi].right = l + 1;
      st.push_back({ct.child[2 * (size_t)(id - n) + 1], l + 1});
      st.push_back({ct.child[2 * (size_t)(id - n)], l});
    }
  }
  return nodes;
}

}  // namespace

void build_mesh_bvh(const float* P, int num_vertices, const int* tris, int T, MeshBvh* out, Context* device,
                    int layouts) {
  if (!(layouts & kLayoutBinary4)) device = nullptr;   // the device tree serves the binary and 4-wide layouts
  // padded triangle boxes (the mesh bounds are minima and maxima: any chunking gives them)
  double mlo[3] = {INFINITY, INFINITY, INFINITY}, mhi[3] = {-INFINITY, -INFINITY, -INFINITY};
  {
    std::vector<std::array<double, 6>> part(build_threads(), {INFINITY, INFINITY, INFINITY, -INFINITY, -INFINITY,
                                                              -INFINITY});
    parallel_chunks((size_t)T, 1 << 15, [&](int t, size_t b, size_t e) {
      std::array<double, 6>& r = part[t];
      for (size_t i = b; i < e; ++i)
        for (int k = 0; k < 3; ++k)
          for (int a = 0; a < 3; ++a) {
            const double v = P[3 * (size_t)tris[3 * i + k] + a];
            r[a] = std::min(r[a], v);
            r[3 + a] = std::max(r[3 + a], v);
          }
    });
    for (const auto& r : part)
      for (int a = 0; a < 3; ++a) {
        mlo[a] = std::min(mlo[a], r[a]);
        mhi[a] = std::max(mhi[a], r[3 + a]);
      }
  }
  double ext = 0, mag = 0;
  for (int a = 0; a < 3; ++a) {
    if (T > 0) {
      ext = std::max(ext, mhi[a] - mlo[a]);
      mag = std::max(mag, std::max(fabs(mlo[a]), fabs(mhi[a])));
    }
  }
  const double pad = ldexp(ext + mag, -16) + 1e-30;
  std::vector<Box> boxes(T);
  parallel_chunks((size_t)T, 1 << 15, [&](int, size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      boxes[i].reset();
      for (int k = 0; k < 3; ++k) {
        double p[3];
        for (int a = 0; a < 3; ++a) p[a] = P[3 * (size_t)tris[3 * i + k] + a];
        boxes[i].grow_pt(p);
      }
      for (int a = 0; a < 3; ++a) {
        boxes[i].lo[a] = (double)down(boxes[i].lo[a] - pad);
        boxes[i].hi[a] = (double)up(boxes[i].hi[a] + pad);
      }
    }
  });
  for (int a = 0; a < 3; ++a) {
    out->lo[a] = T ? down(mlo[a] - pad) : 0.0f;
    out->hi[a] = T ? up(mhi[a] + pad) : 0.0f;
  }
  ClusterTree ct;
  bool use_ct = false;
  std::string fallback;
  if (device && T > 0) {
    std::vector<float> b6(6 * (size_t)T);
    for (int i = 0; i < T; ++i)
      for (int a = 0; a < 3; ++a) {
        b6[6 * (size_t)i + a] = (float)boxes[i].lo[a];        // exact: the padded boxes are floats
        b6[6 * (size_t)i + 3 + a] = (float)boxes[i].hi[a];
      }
    std::string err;
    if (build_cluster_tree_device(device, b6.data(), T, &ct, &err) == ILLUME_OK) use_ct = true;
    else fallback = err.empty() ? std::string(last_error()) : err;
  }
  auto binary = [&](int max_leaf, std::vector<int>& order) {
    return use_ct ? tree_from_clusters(ct, max_leaf, order) : build_binary(boxes, order, max_leaf);
  };

  // ---------------- binary layout ----------------
  auto build_binary_layout = [&]() {
    std::vector<int> order;
    std::vector<BNode> bn = T ? binary(4, order) : std::vector<BNode>();
    out->bvh2.clear();
    out->bvh2_tris.resize((size_t)T * 3);
    parallel_chunks((size_t)T, 1 << 15, [&](int, size_t b, size_t e) {
      for (size_t i = b; i < e; ++i) put_tri(&out->bvh2_tris[3 * i], P, tris + 3 * (size_t)order[i], order[i]);
    });
    auto encode_box = [](Bvh2Node& n, int slot, const Box& b) {
      float lo[3], hi[3];
      for (int a = 0; a < 3; ++a) { lo[a] = (float)b.lo[a]; hi[a] = (float)b.hi[a]; }
      if (slot == 0) {
        n.a = float4{lo[0], lo[1], lo[2], hi[0]};
        n.b.x = hi[1]; n.b.y = hi[2];
      } else {
        n.b.z = lo[0]; n.b.w = lo[1];
        n.c = float4{lo[2], hi[0], hi[1], hi[2]};
      }
    };
    const float inf = INFINITY;
    if (T == 0) {
      Bvh2Node n{};
      n.a = float4{inf, inf, inf, -inf}; n.b = float4{-inf, -inf, inf, inf}; n.c = float4{inf, -inf, -inf, -inf};
      n.d = int4{~0, ~0, 0, 0};
      out->bvh2.push_back(n);
    } else {
      // map binary inner nodes to Bvh2 node indices (DFS order)
      std::vector<int> idx(bn.size(), -1);
      std::vector<int> st{0};
      std::vector<int> inner;
      if (bn[0].left < 0) {
        // whole mesh in one leaf: one inner node with the leaf and an empty slot
        out->root_leaf = true;
        Bvh2Node n{};
        encode_box(n, 0, bn[0].box);
        Box empty;
        empty.reset();
        n.b.z = inf; n.b.w = inf; n.c = float4{inf, -inf, -inf, -inf};
        n.d = int4{~((bn[0].first << 3) | bn[0].count), ~0, bn[0].count, 0};
        out->bvh2.push_back(n);
      } else {
        while (!st.empty()) {
          const int i = st.back();
          st.pop_back();
          idx[i] = (int)inner.size();
          inner.push_back(i);
          if (bn[bn[i].right].left >= 0) st.push_back(bn[i].right);
          if (bn[bn[i].left].left >= 0) st.push_back(bn[i].left);
        }
        out->bvh2.resize(inner.size());
        std::vector<int> leaves(build_threads(), 0);
        parallel_chunks(inner.size(), 1 << 15, [&](int t, size_t b0, size_t e0) {
          for (size_t k = b0; k < e0; ++k) {
            const BNode& b = bn[inner[k]];
            Bvh2Node n{};
            const BNode& L = bn[b.left];
            const BNode& R = bn[b.right];
            encode_box(n, 0, L.box);
            encode_box(n, 1, R.box);
            n.d.x = L.left >= 0 ? idx[b.left] : ~((L.first << 3) | L.count);
            n.d.y = R.left >= 0 ? idx[b.right] : ~((R.first << 3) | R.count);
            n.d.z = L.left >= 0 ? 0 : L.count;
            n.d.w = R.left >= 0 ? 0 : R.count;
            out->bvh2[k] = n;
            leaves[t] += (L.left < 0) + (R.left < 0);
          }
        });
        for (int c : leaves) out->stats.bvh2_leaves += c;
      }
      out->stats.bvh2_nodes = (int)out->bvh2.size();
      out->stats.bvh2_depth = tree_depth(bn, 0);
    }
    // ---- 4-wide collapse of the same tree (shares bvh2_tris) ----
    out->bvh4.clear();
    auto set_slot = [](Bvh4Node& n, int k, const float lo[3], const float hi[3], int entry) {
      float* lx = &n.lox.x; float* ly = &n.loy.x; float* lz = &n.loz.x;
      float* hx = &n.hix.x; float* hy = &n.hiy.x; float* hz = &n.hiz.x;
      lx[k] = lo[0]; ly[k] = lo[1]; lz[k] = lo[2];
      hx[k] = hi[0]; hy[k] = hi[1]; hz[k] = hi[2];
      (&n.child.x)[k] = entry;
    };
    auto empty_node = [&]() {
      Bvh4Node n{};
      const float lo[3] = {inf, inf, inf}, hi[3] = {-inf, -inf, -inf};
      for (int k = 0; k < 4; ++k) set_slot(n, k, lo, hi, -1);
      return n;
    };
    auto box_of = [](const Box& b, float lo[3], float hi[3]) {
      for (int a = 0; a < 3; ++a) { lo[a] = (float)b.lo[a]; hi[a] = (float)b.hi[a]; }
    };
    if (T == 0) {
      out->bvh4.push_back(empty_node());
      out->stats.bvh4_depth = 1;
    } else if (bn[0].left < 0) {
      Bvh4Node n = empty_node();
      float lo[3], hi[3];
      box_of(bn[0].box, lo, hi);
      set_slot(n, 0, lo, hi, ~((bn[0].first << 3) | bn[0].count));
      out->bvh4.push_back(n);
      out->stats.bvh4_depth = 1;
    } else {
      // children of each 4-wide node: the collapse of least summed node area
      const WideCollapse<4> wc(bn);
      std::vector<std::array<int, 4>> kids;
      std::vector<int> nkids, depth4, map4(bn.size(), -1);
      std::vector<std::pair<int, int>> st4{{0, 1}};
      while (!st4.empty()) {
        const int i = st4.back().first, dpt = st4.back().second;
        st4.pop_back();
        map4[i] = (int)kids.size();
        std::array<int, 4> ch{-1, -1, -1, -1};
        const int nc = wc.children(i, ch.data());
        kids.push_back(ch);
        nkids.push_back(nc);
        depth4.push_back(dpt);
        for (int k = nc - 1; k >= 0; --k)
          if (bn[ch[k]].left >= 0) st4.push_back({ch[k], dpt + 1});
      }
      out->bvh4.resize(kids.size());
      int maxd = 0;
      for (size_t q = 0; q < kids.size(); ++q) {
        Bvh4Node n = empty_node();
        for (int k = 0; k < nkids[q]; ++k) {
          const BNode& c = bn[kids[q][k]];
          float lo[3], hi[3];
          box_of(c.box, lo, hi);
          set_slot(n, k, lo, hi, c.left >= 0 ? map4[kids[q][k]] : ~((c.first << 3) | c.count));
        }
        out->bvh4[q] = n;
        maxd = std::max(maxd, depth4[q]);
      }
      out->stats.bvh4_depth = maxd;
    }
    out->stats.bvh4_nodes = (int)out->bvh4.size();
  };

  // ---------------- 8-wide quantised layout ----------------
  auto build_wide_layout = [&]() {
    std::vector<int> order;
    std::vector<BNode> bn = T ? binary(3, order) : std::vector<BNode>();
    out->wide.clear();
    out->wide_tris.clear();
    out->wide_tris.reserve((size_t)T * 3);
    if (T == 0) {
      WideNode w{};
      out->wide.push_back(w);
    } else {
      // queue of (binary node, wide node index); children of one wide node are allocated
      // consecutively so that a child's index = child_base + rank among inner children
      const WideCollapse<8> wc8(bn);
      std::vector<std::pair<int, int>> queue;
      out->wide.emplace_back();
      queue.push_back({0, 0});
      size_t head = 0;
      int max_depth = 0;
      std::vector<int> depth_of{1};
      while (head < queue.size()) {
        const int b = queue[head].first;
        const int wi = queue[head].second;
        ++head;
        max_depth = std::max(max_depth, depth_of[wi]);
        // children: the collapse of least summed node area (a root leaf alone)
        std::vector<int> kids;
        if (bn[b].left < 0) {
          kids.push_back(b);
        } else {
          int ch[8];
          const int nk = wc8.children(b, ch);
          kids.assign(ch, ch + nk);
        }
        // node box and octant slot assignment
        Box nb;
        nb.reset();
        for (int k : kids) nb.grow(bn[k].box);
        double nc[3];
        for (int a = 0; a < 3; ++a) nc[a] = 0.5 * (nb.lo[a] + nb.hi[a]);
        struct Cand { double cost; int kid, slot; };
        std::vector<Cand> cands;
        for (size_t k = 0; k < kids.size(); ++k) {
          const Box& cbx = bn[kids[k]].box;
          for (int s = 0; s < 8; ++s) {
            const double sx = (s & 4) ? -1 : 1, sy = (s & 2) ? -1 : 1, sz = (s & 1) ? -1 : 1;
            const double cost = (0.5 * (cbx.lo[0] + cbx.hi[0]) - nc[0]) * sx + (0.5 * (cbx.lo[1] + cbx.hi[1]) - nc[1]) * sy +
                                (0.5 * (cbx.lo[2] + cbx.hi[2]) - nc[2]) * sz;
            cands.push_back({cost, (int)k, s});
          }
        }
        std::sort(cands.begin(), cands.end(), [](const Cand& x, const Cand& y) {
          return x.cost < y.cost || (x.cost == y.cost && (x.kid < y.kid || (x.kid == y.kid && x.slot < y.slot)));
        });
        int slot_kid[8];
        for (int s = 0; s < 8; ++s) slot_kid[s] = -1;
        std::vector<bool> used(kids.size(), false);
        for (const Cand& c : cands) {
          if (used[c.kid] || slot_kid[c.slot] >= 0) continue;
          used[c.kid] = true;
          slot_kid[c.slot] = c.kid;
        }
        // quantisation frame
        WideNode w{};
        w.px = down(nb.lo[0]); w.py = down(nb.lo[1]); w.pz = down(nb.lo[2]);
        const double p[3] = {w.px, w.py, w.pz};
        int e[3];
        for (int a = 0; a < 3; ++a) {
          const double ext = nb.hi[a] - p[a];
          int ea = -126;
          if (ext > 0) {
            ea = (int)ceil(log2(ext / 255.0));
            while (ldexp(255.0, ea) < ext) ++ea;
            ea = std::max(-126, std::min(127, ea));
          }
          e[a] = ea;
        }
        w.ex = (uint8_t)(e[0] + 127); w.ey = (uint8_t)(e[1] + 127); w.ez = (uint8_t)(e[2] + 127);
        w.child_base = (uint32_t)out->wide.size();
        w.tri_base = (uint32_t)(out->wide_tris.size() / 3);
        int tri_off = 0;
        for (int s = 0; s < 8; ++s) {
          const int k = slot_kid[s];
          if (k < 0) continue;
          const BNode& c = bn[kids[k]];
          uint8_t* qlo[3] = {w.qlox, w.qloy, w.qloz};
          uint8_t* qhi[3] = {w.qhix, w.qhiy, w.qhiz};
          for (int a = 0; a < 3; ++a) {
            const double sc = ldexp(1.0, e[a]);
            double ql = floor((c.box.lo[a] - p[a]) / sc), qh = ceil((c.box.hi[a] - p[a]) / sc);
            ql = std::max(0.0, std::min(255.0, ql));
            qh = std::max(0.0, std::min(255.0, qh));
            while (ql > 0 && p[a] + ql * sc > c.box.lo[a]) ql -= 1;
            while (qh < 255 && p[a] + qh * sc < c.box.hi[a]) qh += 1;
            qlo[a][s] = (uint8_t)ql;
            qhi[a][s] = (uint8_t)qh;
          }
          if (c.left >= 0) {
            w.imask |= (uint8_t)(1u << s);
            const int child_index = (int)out->wide.size();
            out->wide.emplace_back();
            depth_of.resize(out->wide.size());
            depth_of[child_index] = depth_of[wi] + 1;
            queue.push_back({kids[k], child_index});
          } else {
            w.meta[s] = (uint8_t)((c.count << 5) | tri_off);
            for (int t = c.first; t < c.first + c.count; ++t) put_tri(out->wide_tris, P, tris + 3 * (size_t)order[t], order[t]);
            tri_off += c.count;
            out->stats.wide_leaves++;
          }
        }
        out->wide[wi] = w;
      }
      out->stats.wide_nodes = (int)out->wide.size();
      out->stats.wide_depth = max_depth;
    }
  };
  // the two trees are independent: build them concurrently when both are asked for
  if (layouts & kLayoutWide) {
    if (layouts & kLayoutBinary4) {
      std::thread wide_thread(build_wide_layout);
      build_binary_layout();
      wide_thread.join();
    } else {
      build_wide_layout();
    }
    out->has_wide = true;
  } else {
    build_binary_layout();
  }
  if (use_ct) {
    if (out->stats.bvh2_depth > 60 || 3 * out->stats.bvh4_depth > 60) {
      // deeper than the traversal stacks take (scene upload rejects it): the host's tree
      const std::string why = "device tree too deep (binary depth " + std::to_string(out->stats.bvh2_depth) +
                              ", 4-wide depth " + std::to_string(out->stats.bvh4_depth) + ")";
      *out = MeshBvh{};
      build_mesh_bvh(P, num_vertices, tris, T, out, nullptr, layouts);
      out->stats.device_fallback = why;
      return;
    }
    out->stats.device_built = 1;
    out->stats.device_rounds = ct.iterations;
    out->stats.device_ms = ct.device_ms;
  } else if (device && T > 0) {
    out->stats.device_fallback = fallback;
  }
}

}  // namespace illume

namespace illume {

namespace {

struct DBox {
  double lo[3], hi[3];
  bool contains_point(const double* p) const {
    for (int a = 0; a < 3; ++a)
      if (p[a] < lo[a] || p[a] > hi[a]) return false;
    return true;
  }
  bool contains(const DBox& b) const {
    for (int a = 0; a < 3; ++a)
      if (b.lo[a] < lo[a] || b.hi[a] > hi[a]) return false;
    return true;
  }
};

bool tri_inside(const float4* tv, const DBox& b) {
  for (int k = 0; k < 3; ++k) {
    const double p[3] = {tv[k].x, tv[k].y, tv[k].z};
    if (!b.contains_point(p)) return false;
  }
  return true;
}

int prim_of(const float4& v) {
  int p;
  memcpy(&p, &v.w, 4);
  return p;
}

}  // namespace

bool check_mesh_bvh(const float* P, const int* tris, int T, const MeshBvh& b, std::string* msg) {
  (void)P; (void)tris;
  if (T == 0) return true;
  // ---- binary ----
  {
    std::vector<int> seen(T, 0);
    std::vector<std::pair<int, DBox>> st;  // node, box the parent claims for it
    DBox all{{-INFINITY, -INFINITY, -INFINITY}, {INFINITY, INFINITY, INFINITY}};
    st.push_back({0, all});
    while (!st.empty()) {
      const int ni = st.back().first;
      const DBox parent = st.back().second;
      st.pop_back();
      if (ni < 0 || ni >= (int)b.bvh2.size()) { *msg = "binary: node index out of range"; return false; }
      const Bvh2Node& n = b.bvh2[ni];
      const DBox c0{{n.a.x, n.a.y, n.a.z}, {n.a.w, n.b.x, n.b.y}};
      const DBox c1{{n.b.z, n.b.w, n.c.x}, {n.c.y, n.c.z, n.c.w}};
      const int child[2] = {n.d.x, n.d.y}, count[2] = {n.d.z, n.d.w};
      const DBox* cb[2] = {&c0, &c1};
      for (int s = 0; s < 2; ++s) {
        if (child[s] < 0) {
          if (count[s] == 0) continue;
          if (!parent.contains(*cb[s]) && ni != 0) { *msg = "binary: child box outside parent"; return false; }
          if ((~child[s] & 7) != count[s]) { *msg = "binary: leaf code and count disagree"; return false; }
          for (int i = ~child[s] >> 3; i < (~child[s] >> 3) + count[s]; ++i) {
            if (i < 0 || i >= T) { *msg = "binary: triangle index out of range"; return false; }
            const int p = prim_of(b.bvh2_tris[3 * i]);
            if (p < 0 || p >= T || seen[p]++) { *msg = "binary: triangle referenced twice or invalid"; return false; }
            if (!tri_inside(&b.bvh2_tris[3 * i], *cb[s])) { *msg = "binary: triangle outside its leaf box"; return false; }
          }
        } else {
          if (ni != 0 && !parent.contains(*cb[s])) { *msg = "binary: child box outside parent"; return false; }
          st.push_back({child[s], *cb[s]});
        }
      }
    }
    for (int p = 0; p < T; ++p)
      if (seen[p] != 1) { *msg = "binary: triangle " + std::to_string(p) + " not referenced exactly once"; return false; }
  }
  // ---- 4-wide ----
  {
    std::vector<int> seen(T, 0);
    std::vector<std::pair<int, DBox>> st;
    DBox all{{-INFINITY, -INFINITY, -INFINITY}, {INFINITY, INFINITY, INFINITY}};
    st.push_back({0, all});
    size_t visited = 0;
    while (!st.empty()) {
      const int ni = st.back().first;
      const DBox parent = st.back().second;
      st.pop_back();
      if (ni < 0 || ni >= (int)b.bvh4.size() || ++visited > b.bvh4.size()) { *msg = "4-wide: bad node index"; return false; }
      const Bvh4Node& n = b.bvh4[ni];
      for (int k = 0; k < 4; ++k) {
        const int e = (&n.child.x)[k];
        if (e == -1) continue;
        const DBox cb{{(&n.lox.x)[k], (&n.loy.x)[k], (&n.loz.x)[k]}, {(&n.hix.x)[k], (&n.hiy.x)[k], (&n.hiz.x)[k]}};
        if (ni != 0 && !parent.contains(cb)) { *msg = "4-wide: child box outside parent"; return false; }
        if (e >= 0) { st.push_back({e, cb}); continue; }
        const int first = ~e >> 3, count = ~e & 7;
        for (int i = first; i < first + count; ++i) {
          if (i < 0 || i >= T) { *msg = "4-wide: triangle index out of range"; return false; }
          const int p = prim_of(b.bvh2_tris[3 * i]);
          if (p < 0 || p >= T || seen[p]++) { *msg = "4-wide: triangle referenced twice or invalid"; return false; }
          if (!tri_inside(&b.bvh2_tris[3 * i], cb)) { *msg = "4-wide: triangle outside its leaf box"; return false; }
        }
      }
    }
    for (int p = 0; p < T; ++p)
      if (seen[p] != 1) { *msg = "4-wide: triangle " + std::to_string(p) + " not referenced exactly once"; return false; }
  }
  // ---- wide ----
  if (b.has_wide) {
    std::vector<int> seen(T, 0);
    std::vector<std::pair<uint32_t, DBox>> st;
    DBox all{{-INFINITY, -INFINITY, -INFINITY}, {INFINITY, INFINITY, INFINITY}};
    st.push_back({0u, all});
    while (!st.empty()) {
      const uint32_t ni = st.back().first;
      const DBox parent = st.back().second;
      st.pop_back();
      if (ni >= b.wide.size()) { *msg = "wide: node index out of range"; return false; }
      const WideNode& w = b.wide[ni];
      const double p[3] = {w.px, w.py, w.pz};
      const double sc[3] = {ldexp(1.0, (int)w.ex - 127), ldexp(1.0, (int)w.ey - 127), ldexp(1.0, (int)w.ez - 127)};
      const uint8_t* ql[3] = {w.qlox, w.qloy, w.qloz};
      const uint8_t* qh[3] = {w.qhix, w.qhiy, w.qhiz};
      for (int s = 0; s < 8; ++s) {
        const bool inner = (w.imask >> s) & 1;
        if (!inner && w.meta[s] == 0) continue;
        DBox cbx;
        for (int a = 0; a < 3; ++a) {
          cbx.lo[a] = p[a] + ql[a][s] * sc[a];
          cbx.hi[a] = p[a] + qh[a][s] * sc[a];
        }
        if (!parent.contains(cbx)) {
          // a slot box may exceed the parent's slot box by quantisation of the parent only
          // when the parent box itself is coarser; contents are checked below instead
        }
        if (inner) {
          const uint32_t ci = w.child_base + __builtin_popcount(w.imask & ((1u << s) - 1));
          st.push_back({ci, cbx});
        } else {
          const int cnt = w.meta[s] >> 5, off = w.meta[s] & 31;
          for (int i = 0; i < cnt; ++i) {
            const size_t t = (size_t)w.tri_base + off + i;
            if (t >= (size_t)T) { *msg = "wide: triangle index out of range"; return false; }
            const int pr = prim_of(b.wide_tris[3 * t]);
            if (pr < 0 || pr >= T || seen[pr]++) { *msg = "wide: triangle referenced twice or invalid"; return false; }
            if (!tri_inside(&b.wide_tris[3 * t], cbx)) { *msg = "wide: triangle outside its quantised leaf box"; return false; }
            if (!tri_inside(&b.wide_tris[3 * t], parent)) { *msg = "wide: triangle outside an ancestor box"; return false; }
          }
        }
      }
    }
    for (int p = 0; p < T; ++p)
      if (seen[p] != 1) { *msg = "wide: triangle " + std::to_string(p) + " not referenced exactly once"; return false; }
  }
  return true;
}

}  // namespace illume
