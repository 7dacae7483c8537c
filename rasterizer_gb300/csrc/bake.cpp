// Host-side occluder preparation: quad decomposition, SAH batching and the
// 11/11/10 occluder bake.  The output must be byte-identical to the
// reference's (the rasteriser is bit-exact only on identical packed input),
// so each routine follows the steps of its reference counterpart:
//   decompose        QuadDecomposition.cpp:326-445 (+ Edmonds matching :28-309)
//   generateBatches  SurfaceAreaHeuristic.cpp:10-104
//   bake             Occluder.cpp:7-181
// All float math goes through x86_emu.cuh (separately rounded, x86 NaN rules,
// RSQRTPS from the measured table), so the result is the same on x86-64 and
// aarch64 hosts.
#include <algorithm>
#include <cstdint>
#include <cstring>
#include <future>
#include <limits>
#include <queue>
#include <string>
#include <system_error>
#include <thread>
#include <utility>
#include <vector>

#include "../../include/rasterizer_gb300.h"
#include "bake_math.cuh"
#include "x86_emu.cuh"

namespace {

using namespace x86;
using bake::V4;
using bake::vadd;
using bake::vsub;
using bake::normalize;

V4 load4(const float* p)
{
  V4 r;
  std::memcpy(r.v, p, 16);
  return r;
}

// COMISS-based predicates: false when unordered
bool gt_ss(float a, float b) { return a > b; }
bool ge_ss(float a, float b) { return a >= b; }
bool lt_ss(float a, float b) { return a < b; }

struct Box {
  V4 lo, hi;
  Box()
  {
    for (int i = 0; i < 4; ++i) {
      lo.v[i] = std::numeric_limits<float>::infinity();
      hi.v[i] = -std::numeric_limits<float>::infinity();
    }
  }
  void grow(const V4& p)
  {
    for (int i = 0; i < 4; ++i) {
      lo.v[i] = xmin(lo.v[i], p.v[i]);
      hi.v[i] = xmax(hi.v[i], p.v[i]);
    }
  }
  void grow(const Box& b)
  {
    for (int i = 0; i < 4; ++i) {
      lo.v[i] = xmin(lo.v[i], b.lo.v[i]);
      hi.v[i] = xmax(hi.v[i], b.hi.v[i]);
    }
  }
  float center2(int axis) const { return xadd(lo.v[axis], hi.v[axis]); }
  // dot(e, e.yzx) over xyz: (ex*ey + ey*ez) + (ez*ex + 0)
  float area() const
  {
    const float e[4] = {xsub(hi.v[0], lo.v[0]), xsub(hi.v[1], lo.v[1]), xsub(hi.v[2], lo.v[2]),
                        xsub(hi.v[3], lo.v[3])};
    const float f[4] = {e[1], e[2], e[0], e[3]};
    return dp3(e, f);
  }
};

// ---- maximum matching on the triangle adjacency graph -----------------------------
// Edmonds' blossom algorithm with the search order of QuadDecomposition.cpp:28-309:
// a greedy maximal matching in vertex order, then one breadth-first augmenting
// path search per still-unmatched vertex, blossoms kept in a union-find forest
// that is invalidated by bumping a per-search stamp.
// Triangle adjacency in compressed rows: the neighbours of v are
// nbr[off[v] .. off[v+1]), in the order the graph construction found them.
struct Adjacency {
  std::vector<uint32_t> off;
  std::vector<int> nbr;
  struct Row {
    const int* b;
    const int* e;
    const int* begin() const { return b; }
    const int* end() const { return e; }
  };
  size_t size() const { return off.empty() ? 0 : off.size() - 1; }
  Row operator[](int v) const { return Row{nbr.data() + off[v], nbr.data() + off[v + 1]}; }
};

class BlossomMatcher {
 public:
  explicit BlossomMatcher(const Adjacency& adj)
      : adj_(adj), mate_(adj.size(), -1), bridge_(adj.size()), node_(adj.size())
  {
    const int n = (int)adj.size();
    std::vector<int> open;
    for (int v = 0; v < n; ++v) {
      if (mate_[v] != -1) continue;
      bool paired = false;
      for (int w : adj_[v])
        if (mate_[w] == -1) {
          pair(v, w);
          paired = true;
          break;
        }
      if (!paired) open.push_back(v);
    }
    std::vector<int> path;
    for (int v : open) {
      if (mate_[v] != -1) continue;
      if (search(v, path)) {
        for (size_t i = 0; i < path.size(); i += 2) pair(path[i], path[i + 1]);
        path.clear();
      }
    }
  }

  int mate(int v) const { return mate_[v]; }

 private:
  struct Node {
    int depth = 0, parent = -1, base = 0, stamp = 0;
  };

  void pair(int v, int w)
  {
    mate_[v] = w;
    mate_[w] = v;
  }

  int root_of(int x)
  {
    if (node_[x].stamp != stamp_) return x;
    if (x != node_[x].base) node_[x].base = root_of(node_[x].base);
    return node_[x].base;
  }

  void join(int x, int y)
  {
    const int rx = root_of(x);
    node_[rx].base = root_of(y);
  }

  void make_root(int x)
  {
    const int rx = root_of(x);
    node_[rx].base = x;
    node_[x].base = x;
  }

  bool search(int root, std::vector<int>& path)
  {
    ++stamp_;
    node_[root].depth = 0;
    node_[root].parent = -1;
    node_[root].stamp = stamp_;
    node_[root].base = root;
    frontier_.push(root);
    while (!frontier_.empty()) {
      const int v = frontier_.front();
      frontier_.pop();
      for (int w : adj_[v]) {
        if (visit(root, v, w, path)) {
          while (!frontier_.empty()) frontier_.pop();
          return true;
        }
      }
    }
    return false;
  }

  bool visit(int root, int v, int w, std::vector<int>& path)
  {
    const int vb = root_of(v), wb = root_of(w);
    if (vb == wb) return false;
    if (node_[wb].stamp != stamp_) {
      if (mate_[w] == -1) {
        path.push_back(w);
        trace(v, root, path);
        return true;
      }
      grow(v, w);
    } else if (node_[wb].depth % 2 == 0) {
      contract(v, w);
    }
    return false;
  }

  void grow(int v, int w)
  {
    const int u = mate_[w];
    node_[w].depth = node_[v].depth + 1 + (node_[v].depth & 1);
    node_[w].parent = v;
    node_[w].stamp = stamp_;
    node_[w].base = w;
    node_[u].depth = node_[w].depth + 1;
    node_[u].parent = w;
    node_[u].stamp = stamp_;
    node_[u].base = u;
    frontier_.push(u);
  }

  void contract(int v, int w)
  {
    const int b = common_ancestor(v, w);
    contract_path(b, v, w);
    contract_path(b, w, v);
  }

  void contract_path(int b, int v, int w)
  {
    int u = root_of(v);
    while (u != b) {
      join(b, u);
      u = mate_[u];
      join(b, u);
      make_root(b);
      frontier_.push(u);
      bridge_[u] = std::make_pair(v, w);
      u = root_of(node_[u].parent);
    }
  }

  int common_ancestor(int v, int w)
  {
    while (w != v) {
      if (node_[v].depth > node_[w].depth) v = node_[v].parent;
      else w = node_[w].parent;
    }
    return root_of(v);
  }

  // alternating path from s back to t (appends to path)
  void trace(int s, int t, std::vector<int>& path)
  {
    if (s == t) {
      path.push_back(s);
    } else if (node_[s].depth % 2 == 0) {
      path.push_back(s);
      path.push_back(mate_[s]);
      trace(node_[mate_[s]].parent, t, path);
    } else {
      const int v = bridge_[s].first, w = bridge_[s].second;
      path.push_back(s);
      const size_t from = path.size();
      trace(v, mate_[s], path);
      std::reverse(path.begin() + (std::ptrdiff_t)from, path.end());
      trace(w, t, path);
    }
  }

  const Adjacency& adj_;
  std::vector<int> mate_;
  std::vector<std::pair<int, int>> bridge_;
  std::vector<Node> node_;
  std::queue<int> frontier_;
  int stamp_ = 0;
};

// Two triangles (v0,v1,v2) and (v2,v3,v0) may form a quad if v1 and v3 lie
// within 0.5 units of the other triangle's plane (QuadDecomposition.cpp:326-343).
bool mergeable(const V4& v0, const V4& v1, const V4& v2, const V4& v3)
{
  const float maxDepthError = 0.5f;
  const V4 n0 = normalize(tri_normal(v0, v1, v2));
  const V4 n2 = normalize(tri_normal(v2, v3, v0));
  const V4 d = vsub(v1, v3);
  const float a = fabs_(dp3(n0.v, d.v));
  const float b = fabs_(dp3(n2.v, d.v));
  return !(gt_ss(a, maxDepthError) || gt_ss(b, maxDepthError));
}

// The directed edges of all triangles grouped by their first vertex; within a
// group in (triangle, edge) order, i.e. the order in which the reference's
// edge map receives them (QuadDecomposition.cpp:357-372).
struct EdgeTable {
  std::vector<uint32_t> start;  // per vertex: first entry of its group
  std::vector<uint32_t> to;     // per entry: second vertex of the edge
  std::vector<uint32_t> tri;    // per entry: triangle
  std::vector<uint32_t> apex;   // per entry: the triangle's third vertex

  EdgeTable(const uint32_t* idx, uint32_t triCount, uint32_t numVerts)
      : start(numVerts + 1, 0), to(3 * (size_t)triCount), tri(3 * (size_t)triCount), apex(3 * (size_t)triCount)
  {
    for (size_t k = 0; k < 3 * (size_t)triCount; ++k) ++start[idx[k] + 1];
    for (uint32_t v = 0; v < numVerts; ++v) start[v + 1] += start[v];
    std::vector<uint32_t> cur(start.begin(), start.end() - 1);
    for (uint32_t t = 0; t < triCount; ++t)
      for (int e = 0; e < 3; ++e) {
        const uint32_t a = idx[3 * t + e], b = idx[3 * t + (e + 1) % 3], c = idx[3 * t + (e + 2) % 3];
        const uint32_t k = cur[a]++;
        to[k] = b;
        tri[k] = t;
        apex[k] = c;
      }
  }
};

std::vector<uint32_t> decompose(const uint32_t* idx, uint32_t nIdx, const float* verts)
{
  const uint32_t triCount = nIdx / 3;
  uint32_t numVerts = 0;
  for (uint32_t k = 0; k < nIdx; ++k) numVerts = std::max(numVerts, idx[k] + 1);
  const EdgeTable E(idx, triCount, numVerts);
  auto vtx = [&](uint32_t i) { return load4(verts + 4 * (size_t)i); };
  // Mergeable neighbours, in the order the reference's loop finds them: for
  // each triangle t (after its own edges entered the map), each edge e, the
  // triangles t' <= t holding the reverse edge, in map order.  A triangle with
  // a repeated vertex holds an edge and its reverse; the reference then makes
  // it its own neighbour, may match it with itself, and its augmenting search
  // can then walk a parent chain that never ends (or the triangle is dropped
  // from the output).  Here a triangle is never its own neighbour: the result
  // is the reference's wherever the reference does not match a triangle with
  // itself, and such a triangle is matched with another or emitted alone.
  std::vector<std::pair<uint32_t, uint32_t>> found;
  for (uint32_t t = 0; t < triCount; ++t) {
    const uint32_t i[3] = {idx[3 * t], idx[3 * t + 1], idx[3 * t + 2]};
    for (int e = 0; e < 3; ++e) {
      const uint32_t a = i[(e + 1) % 3], b = i[e];  // the shared edge runs the other way: a -> b
      for (uint32_t k = E.start[a]; k < E.start[a + 1] && E.tri[k] <= t; ++k) {
        if (E.to[k] != b || E.tri[k] == t) continue;
        if (mergeable(vtx(i[e]), vtx(E.apex[k]), vtx(i[(e + 1) % 3]), vtx(i[(e + 2) % 3])))
          found.emplace_back(t, E.tri[k]);
      }
    }
  }
  Adjacency adj;
  adj.off.assign((size_t)triCount + 1, 0);
  for (const auto& pr : found) {
    ++adj.off[pr.first + 1];
    ++adj.off[pr.second + 1];
  }
  for (uint32_t t = 0; t < triCount; ++t) adj.off[t + 1] += adj.off[t];
  adj.nbr.resize(adj.off[triCount]);
  {
    std::vector<uint32_t> cur(adj.off.begin(), adj.off.end() - 1);
    for (const auto& pr : found) {
      adj.nbr[cur[pr.first]++] = (int)pr.second;
      adj.nbr[cur[pr.second]++] = (int)pr.first;
    }
  }
  BlossomMatcher matching(adj);
  std::vector<uint32_t> out;
  out.reserve((size_t)triCount * 4);
  for (uint32_t t = 0; t < triCount; ++t) {
    const int m = matching.mate((int)t);
    const uint32_t i[3] = {idx[3 * t], idx[3 * t + 1], idx[3 * t + 2]};
    if (m == -1) {
      out.insert(out.end(), {i[0], i[2], i[1], i[0]});  // lone triangle as a degenerate quad
      continue;
    }
    if (t >= (uint32_t)m) continue;  // emitted with the lower-numbered triangle
    bool done = false;
    for (int e = 0; e < 3 && !done; ++e) {
      const uint32_t a = i[(e + 1) % 3], b = i[e];
      for (uint32_t k = E.start[a]; k < E.start[a + 1]; ++k)
        if (E.to[k] == b && E.tri[k] == (uint32_t)m) {
          out.insert(out.end(), {i[e], i[(e + 2) % 3], i[(e + 1) % 3], E.apex[k]});
          done = true;
          break;
        }
    }
  }
  return out;
}

// ---- SAH batching -------------------------------------------------------------------

// Stable sort of the indices [begin, end) by c[index] under `<`, for keys
// without NaN: an LSD radix sort (three passes of 11, 11, 10 bits) of the keys
// mapped to unsigned integers in float order, both zeros mapped alike (`<`
// ties them, so stability keeps their order).  The same permutation as
// std::stable_sort with that comparison.
void stable_sort_by_key(uint32_t* begin, uint32_t* end, const float* c, std::vector<uint64_t>& a,
                        std::vector<uint64_t>& b)
{
  const size_t n = (size_t)(end - begin);
  a.resize(n);
  b.resize(n);
  for (size_t i = 0; i < n; ++i) {
    uint32_t u = c[begin[i]] == 0.0f ? 0u : fu(c[begin[i]]);
    u = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
    a[i] = ((uint64_t)u << 32) | begin[i];
  }
  const int shifts[3] = {32, 43, 54}, bits[3] = {11, 11, 10};
  for (int pass = 0; pass < 3; ++pass) {
    const uint32_t mask = (1u << bits[pass]) - 1u;
    std::vector<size_t> cnt((size_t)mask + 2, 0);
    for (size_t i = 0; i < n; ++i) ++cnt[((a[i] >> shifts[pass]) & mask) + 1];
    for (size_t d = 0; d <= mask; ++d) cnt[d + 1] += cnt[d];
    for (size_t i = 0; i < n; ++i) b[cnt[(a[i] >> shifts[pass]) & mask]++] = a[i];
    a.swap(b);
  }
  for (size_t i = 0; i < n; ++i) begin[i] = (uint32_t)a[i];
}

void sort_by_axis(uint32_t* begin, uint32_t* end, const float* c, bool ctrNaN)
{
  static thread_local std::vector<uint64_t> ta, tb;
  if (!ctrNaN && end - begin >= 2048) stable_sort_by_key(begin, end, c, ta, tb);
  else std::stable_sort(begin, end, [c](uint32_t x, uint32_t y) { return c[x] < c[y]; });
}

// ctr[axis][i]: box i's centre along the axis (times two), computed once; the
// sorts compare these floats exactly as the reference compares the centres.
int sah_split(const std::vector<Box>& boxes, const std::vector<float> (&ctr)[3], bool ctrNaN, uint32_t gran,
              uint32_t* begin, uint32_t* end)
{
  const uint32_t n = (uint32_t)(end - begin);
  float bestCost = std::numeric_limits<float>::infinity();
  int bestAxis = -1, bestIndex = -1;
  std::vector<float> left(n), right(n);
  for (int axis = 0; axis < 3; ++axis) {
    sort_by_axis(begin, end, ctr[axis].data(), ctrNaN);
    Box acc;
    for (uint32_t i = 0; i < n; ++i) {
      acc.grow(boxes[begin[i]]);
      left[i] = acc.area();
    }
    Box acc2;
    for (int i = (int)n - 1; i >= 0; --i) {
      acc2.grow(boxes[begin[i]]);
      right[i] = acc2.area();
    }
    for (uint32_t s = gran; s < n - gran; s += gran) {
      const float cost = xadd(xmul(left[s - 1], i2f((int32_t)s)), xmul(right[s], i2f((int32_t)(n - s))));
      if (lt_ss(cost, bestCost)) {
        bestCost = cost;
        bestAxis = axis;
        bestIndex = (int)s;
      }
    }
  }
  if (bestAxis < 0) return -1;
  // without NaN centres the range is still in the order of the last axis
  // sorted, and sorting it again by that axis changes nothing
  if (bestAxis != 2 || ctrNaN) sort_by_axis(begin, end, ctr[bestAxis].data(), ctrNaN);
  return bestIndex;
}

void sah_recurse(const std::vector<Box>& boxes, const std::vector<float> (&ctr)[3], bool ctrNaN, uint32_t target,
                 uint32_t gran, uint32_t* begin, uint32_t* end, std::vector<std::vector<uint32_t>>& out)
{
  // The reference's split search needs more than two split granules (its loop
  // bound is unsigned), and a split must exist; otherwise keep the range whole.
  const int split = (size_t)(end - begin) > 2 * (size_t)gran ? sah_split(boxes, ctr, ctrNaN, gran, begin, end) : -1;
  if (split < 0) {
    out.emplace_back(begin, end);
    return;
  }
  uint32_t* range[3] = {begin, begin + split, end};
  auto half = [&](int i, std::vector<std::vector<uint32_t>>& dst) {
    if ((size_t)(range[i + 1] - range[i]) < target) dst.emplace_back(range[i], range[i + 1]);
    else sah_recurse(boxes, ctr, ctrNaN, target, gran, range[i], range[i + 1], dst);
  };
  // Large halves are independent (disjoint index ranges, read-only boxes):
  // the first runs on another thread, and its batches still come first.
  constexpr size_t kParallelMin = 32768;
  if (split >= (int)kParallelMin && (size_t)(end - begin) - (size_t)split >= kParallelMin) {
    std::vector<std::vector<uint32_t>> first;
    std::future<void> job;
    try {
      job = std::async(std::launch::async, [&] { half(0, first); });
    } catch (const std::system_error&) {  // no thread to be had: in sequence
      half(0, first);
    }
    std::vector<std::vector<uint32_t>> second;
    half(1, second);
    if (job.valid()) job.get();
    for (auto* part : {&first, &second})
      for (auto& b : *part) out.push_back(std::move(b));
    return;
  }
  for (int i = 0; i < 2; ++i) half(i, out);
}

}  // namespace

extern "C" {

int occ_quad_decompose(const uint32_t* indices, uint32_t nIndices, const float* vertices, uint32_t nVertices,
                       uint32_t* out, uint32_t* outCount)
{
  if (!indices || !vertices || !out || !outCount || nIndices % 3) return OCC_ERR_INVALID_ARG;
  for (uint32_t i = 0; i < nIndices; ++i)
    if (indices[i] >= nVertices) return OCC_ERR_INVALID_ARG;
  std::vector<uint32_t> q = decompose(indices, nIndices, vertices);
  std::copy(q.begin(), q.end(), out);
  *outCount = (uint32_t)q.size();
  return OCC_OK;
}

int occ_sah_generate_batches(const float* aabbs, uint32_t n, uint32_t targetSize, uint32_t splitGranularity,
                             uint32_t* flat, uint32_t* offsets, uint32_t* numBatches)
{
  if (!aabbs || !flat || !offsets || !numBatches || !splitGranularity) return OCC_ERR_INVALID_ARG;
  // The reference's split search needs more than two split granules (its loop
  // bound n - granularity is unsigned); smaller inputs form a single batch here.
  if (n <= 2 * splitGranularity) {
    for (uint32_t i = 0; i < n; ++i) flat[i] = i;
    offsets[0] = 0;
    offsets[1] = n;
    *numBatches = n ? 1 : 0;
    return OCC_OK;
  }
  std::vector<Box> boxes(n);
  for (uint32_t i = 0; i < n; ++i) {
    boxes[i].lo = load4(aabbs + 8 * (size_t)i);
    boxes[i].hi = load4(aabbs + 8 * (size_t)i + 4);
  }
  std::vector<uint32_t> order(n);
  for (uint32_t i = 0; i < n; ++i) order[i] = i;
  std::vector<std::vector<uint32_t>> batches;
  std::vector<float> ctr[3];
  bool ctrNaN = false;
  for (int axis = 0; axis < 3; ++axis) {
    ctr[axis].resize(n);
    for (uint32_t i = 0; i < n; ++i) {
      ctr[axis][i] = boxes[i].center2(axis);
      ctrNaN |= ctr[axis][i] != ctr[axis][i];
    }
  }
  sah_recurse(boxes, ctr, ctrNaN, targetSize, splitGranularity, order.data(), order.data() + n, batches);
  uint32_t pos = 0;
  for (size_t b = 0; b < batches.size(); ++b) {
    offsets[b] = pos;
    for (uint32_t q : batches[b]) flat[pos++] = q;
  }
  offsets[batches.size()] = pos;
  *numBatches = (uint32_t)batches.size();
  return OCC_OK;
}

int occ_occluder_bake(const float* vertices, uint32_t nVertices, const float refMin[4], const float refMax[4],
                      uint32_t* packedOut, uint32_t* packetCount, float boundsMin[4], float boundsMax[4],
                      float center[4])
{
  if (!vertices || !refMin || !refMax || !packedOut || !packetCount || !boundsMin || !boundsMax || !center)
    return OCC_ERR_INVALID_ARG;
  // whole packets of 8 quads: the reference asserts a multiple of 16 vertices
  // (Occluder.cpp:9) but packs 32 at a time (:108-122) and reads past its
  // array for the other half of those counts
  if (nVertices == 0 || nVertices % 32 != 0) return OCC_ERR_INVALID_ARG;
  const uint32_t nq = nVertices / 4;
  auto vtx = [&](uint32_t i) { return load4(vertices + 4 * (size_t)i); };

  // k-means of the quad normals around the six axis directions (Occluder.cpp:11-78)
  std::vector<V4> normals(nq);
  for (uint32_t q = 0; q < nq; ++q) normals[q] = bake::quad_normal(vtx(4 * q), vtx(4 * q + 1), vtx(4 * q + 2), vtx(4 * q + 3));
  V4 centroid[6];
  for (int k = 0; k < 6; ++k) centroid[k] = bake::seed_centroid(k);
  std::vector<uint32_t> cluster(nq, 0);
  bool changed = true;
  for (int iter = 0; iter < 10 && changed; ++iter) {
    changed = false;
    for (uint32_t q = 0; q < nq; ++q) {
      float best = -std::numeric_limits<float>::infinity();
      uint32_t bestK = 0;
      for (uint32_t k = 0; k < 6; ++k) {
        const float d = dp3(centroid[k].v, normals[q].v);
        if (ge_ss(d, best)) {
          best = d;
          bestK = k;
        }
      }
      if (cluster[q] != bestK) {
        cluster[q] = bestK;
        changed = true;
      }
    }
    for (auto& c : centroid) c = V4{{0, 0, 0, 0}};
    for (uint32_t q = 0; q < nq; ++q) centroid[cluster[q]] = vadd(centroid[cluster[q]], normals[q]);
    for (auto& c : centroid) c = normalize(c);
  }
  std::vector<uint32_t> order;  // quads grouped by cluster, original order within
  order.reserve(nq);
  for (uint32_t k = 0; k < 6; ++k)
    for (uint32_t q = 0; q < nq; ++q)
      if (cluster[q] == k) order.push_back(q);

  // 11/11/10 quantisation in the reference box (Occluder.cpp:97-157)
  const V4 lo = load4(refMin), hi = load4(refMax);
  V4 inv;
  for (int i = 0; i < 4; ++i) inv.v[i] = xdiv(1.0f, xsub(hi.v[i], lo.v[i]));
  uint32_t packets = 0;
  for (uint32_t g = 0; g < nq; g += 8) {
    for (uint32_t j = 0; j < 4; ++j) {
      for (uint32_t l = 0; l < 8; ++l)
        packedOut[(size_t)packets * 8 + 8 * j + l] = bake::pack_vertex(vtx(4 * order[g + l] + j), lo, inv);
    }
    packets += 4;
  }
  *packetCount = packets;

  // bounds over the input vertices, w = 1 (Occluder.cpp:162-178)
  V4 mn, mx;
  for (int i = 0; i < 4; ++i) {
    mn.v[i] = std::numeric_limits<float>::infinity();
    mx.v[i] = -std::numeric_limits<float>::infinity();
  }
  for (uint32_t i = 0; i < nVertices; ++i) {
    const V4 p = vtx(i);
    for (int a = 0; a < 4; ++a) {
      mn.v[a] = xmin(p.v[a], mn.v[a]);
      mx.v[a] = xmax(p.v[a], mx.v[a]);
    }
  }
  mn.v[3] = 1.0f;
  mx.v[3] = 1.0f;
  for (int a = 0; a < 4; ++a) {
    boundsMin[a] = mn.v[a];
    boundsMax[a] = mx.v[a];
    center[a] = xmul(xadd(mx.v[a], mn.v[a]), 0.5f);
  }
  return OCC_OK;
}

// The demo's scene preparation in one call (Main.cpp:86-128): quads,
// padding to whole packets with the first quad, per-quad boxes, SAH batches,
// the reference box of all vertices, one Occluder::bake per batch (batches
// baked on several threads, each into its own part of the output).
int occ_scene_bake(const float* vertices, uint32_t nVertices, const uint32_t* indices, uint32_t nIndices,
                   uint32_t targetSize, uint32_t splitGranularity, uint32_t capacityCount, uint64_t capacityWords,
                   uint32_t* count, uint64_t* words, uint32_t* packetCounts, uint32_t* packed, float* bounds)
{
  if ((!vertices && nVertices) || (!indices && nIndices) || !count || !words || nIndices % 3 || !splitGranularity)
    return OCC_ERR_INVALID_ARG;
  std::vector<uint32_t> q(4 * (size_t)(nIndices / 3) + 4);
  uint32_t nqIdx = 0;
  if (nIndices) {
    const int st = occ_quad_decompose(indices, nIndices, vertices, nVertices, q.data(), &nqIdx);
    if (st != OCC_OK) return st;
  }
  q.resize(nqIdx);
  while (!q.empty() && q.size() % 32) q.push_back(q[0]);  // Main.cpp:94-98
  const uint32_t nq = (uint32_t)(q.size() / 4);
  auto vtx = [&](uint32_t i) { return load4(vertices + 4 * (size_t)i); };
  std::vector<float> boxes(8 * (size_t)nq);
  for (uint32_t k = 0; k < nq; ++k) {
    Box b;
    for (int c = 0; c < 4; ++c) b.grow(vtx(q[4 * (size_t)k + c]));  // Main.cpp:100-107
    std::memcpy(&boxes[8 * (size_t)k], b.lo.v, 16);
    std::memcpy(&boxes[8 * (size_t)k + 4], b.hi.v, 16);
  }
  std::vector<uint32_t> flat(std::max<uint32_t>(nq, 1)), offs((size_t)nq + 2);
  uint32_t nb = 0;
  if (nq) {
    const int st = occ_sah_generate_batches(boxes.data(), nq, targetSize, splitGranularity, flat.data(), offs.data(), &nb);
    if (st != OCC_OK) return st;
  }
  Box ref;  // Main.cpp:109-113
  for (uint32_t i = 0; i < nVertices; ++i) ref.grow(vtx(i));
  std::vector<uint64_t> wordStart((size_t)nb + 1, 0);
  for (uint32_t b = 0; b < nb; ++b) wordStart[b + 1] = wordStart[b] + 4ull * (offs[b + 1] - offs[b]);  // a word per vertex
  *count = nb;
  *words = wordStart[nb];
  if (!packetCounts && !packed && !bounds) return OCC_OK;  // sizes only
  if (!packetCounts || !packed || !bounds) return OCC_ERR_INVALID_ARG;
  if (nb > capacityCount || wordStart[nb] > capacityWords) return OCC_ERR_CAPACITY;
  // one Occluder::bake per batch; contiguous runs of batches per thread
  std::vector<int> status(nb, OCC_OK);
  auto bakeRange = [&](uint32_t b0, uint32_t b1) {
    std::vector<float> v;
    for (uint32_t b = b0; b < b1; ++b) {
      v.resize(16 * (size_t)(offs[b + 1] - offs[b]));
      size_t o = 0;
      for (uint32_t k = offs[b]; k < offs[b + 1]; ++k)
        for (int c = 0; c < 4; ++c, o += 4) std::memcpy(&v[o], vertices + 4 * (size_t)q[4 * (size_t)flat[k] + c], 16);
      float* B = bounds + 20 * (size_t)b;
      std::memcpy(B, ref.lo.v, 16);
      std::memcpy(B + 4, ref.hi.v, 16);
      status[b] = occ_occluder_bake(v.data(), (uint32_t)(v.size() / 4), B, B + 4, packed + wordStart[b],
                                    &packetCounts[b], B + 8, B + 12, B + 16);
    }
  };
  const uint32_t hw = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  const uint32_t tasks = std::min<uint32_t>(hw, std::max<uint32_t>(1, nb / 64));
  std::vector<std::future<void>> jobs;
  for (uint32_t t = 1; t < tasks; ++t) {
    const uint32_t b0 = (uint32_t)((uint64_t)nb * t / tasks), b1 = (uint32_t)((uint64_t)nb * (t + 1) / tasks);
    try {
      jobs.push_back(std::async(std::launch::async, bakeRange, b0, b1));
    } catch (const std::system_error&) {  // no thread to be had: in sequence
      bakeRange(b0, b1);
    }
  }
  bakeRange(0, (uint32_t)((uint64_t)nb / tasks));
  for (auto& j : jobs) j.get();
  for (int st : status)
    if (st != OCC_OK) return st;
  return OCC_OK;
}

}  // extern "C"
