// Checks of the quantised 4-wide node encoding (rtgb::convert_bvh) on the
// CPU, for scenes at awkward scales and offsets:
//
//   encode  every child slot's planes p + q * 2^e enclose the exact bounds of
//           the primitives under it (exact comparisons through error-free
//           float expansions);
//   visit   the kernels' node-visit arithmetic (trace_core.cuh,
//           visit_wide_stk), restated op for op in binary32 with fmaf, gives
//           an interval [near, far] that contains the ray's whole exact
//           entry-exit interval of the child's exact bounds, at each node on
//           the path from the root to a random triangle (rays from outside
//           and inside the scene, a quarter with a direction component of 0).
//
// Prints "ok <scene> <nodes> <paths>" per scene or "FAIL ..." and exits 1.
// Built with -ffp-contract=off so that no operation is fused unless written
// as fmaf.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "rt_internal.h"

using namespace rtgb;

namespace {

int g_fail = 0;

void fail(const std::string& what) {
  if (g_fail < 20) std::printf("FAIL %s\n", what.c_str());
  ++g_fail;
}

// Shewchuk's GROW-EXPANSION with Knuth's two-sum: the exact sum of doubles
// as nonoverlapping components; its sign is the sign of the largest one.
void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  const double bb = s - a;
  e = (a - (s - bb)) + (b - bb);
}
int exact_sign(std::initializer_list<double> terms) {
  std::vector<double> ex;
  for (double t : terms) {
    double q = t;
    std::vector<double> nx;
    for (double c : ex) {
      double s, e;
      two_sum(q, c, s, e);
      if (e != 0.0) nx.push_back(e);
      q = s;
    }
    if (q != 0.0) nx.push_back(q);
    ex.swap(nx);
  }
  for (size_t k = ex.size(); k-- > 0;)
    if (ex[k] != 0.0) return ex[k] > 0.0 ? 1 : -1;
  return 0;
}

float f_of(uint32_t u) {
  float f;
  std::memcpy(&f, &u, 4);
  return f;
}
uint32_t u_of(float f) {
  uint32_t u;
  std::memcpy(&u, &f, 4);
  return u;
}

struct Box {
  double lo[3] = {INFINITY, INFINITY, INFINITY}, hi[3] = {-INFINITY, -INFINITY, -INFINITY};
  void grow(const Box& b) {
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::fmin(lo[a], b.lo[a]);
      hi[a] = std::fmax(hi[a], b.hi[a]);
    }
  }
};

struct Scene {
  std::string name;
  std::vector<RtTriangle64> tris;
};

std::vector<RtTriangle64> soup(uint32_t seed, uint32_t n, double side, double sigma, const double off[3],
                               bool flat_z = false) {
  std::mt19937_64 g(seed);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  std::normal_distribution<double> nd(0.0, 1.0);
  std::vector<RtTriangle64> t(n);
  for (auto& tr : t) {
    std::memset(&tr, 0, sizeof(tr));
    double c[3] = {u(g) * side, u(g) * side, u(g) * side};
    float* vs[3] = {tr.v0, tr.v1, tr.v2};
    for (auto* v : vs)
      for (int k = 0; k < 3; ++k) v[k] = (float)(off[k] + c[k] + sigma * nd(g));
    if (flat_z)
      for (auto* v : vs) v[2] = (float)off[2];
  }
  return t;
}

// The node visit of the kernels for one child slot, binary32.
void visit_child(const float* node, int j, const float o[3], const float d[3], float cull_lo, float cull_hi,
                 float& n_out, float& f_out) {
  const float eps = 5.42101086242752217e-20f;  // 2^-64
  float ix[3];
  for (int a = 0; a < 3; ++a) ix[a] = 1.0f / (std::fabs(d[a]) > eps ? d[a] : std::copysign(eps, d[a]));
  const float scale[3] = {node[3], node[14], node[15]};
  const uint32_t qw[6] = {u_of(node[8]), u_of(node[9]), u_of(node[10]), u_of(node[11]), u_of(node[12]),
                          u_of(node[13])};
  const float widen = 9.5367431640625e-07f;  // 2^-20
  float tn[3], tf[3];
  for (int a = 0; a < 3; ++a) {
    const float A = scale[a] * ix[a];
    const float B = (node[a] - o[a]) * ix[a];
    const float C = B - A;
    const float M = std::fabs(B) + std::fabs(A);
    const float cn = std::fmaf(M, -widen, C), cf = std::fmaf(M, widen, C);
    const uint32_t wn = ix[a] >= 0.0f ? qw[2 * a] : qw[2 * a + 1], wf = ix[a] >= 0.0f ? qw[2 * a + 1] : qw[2 * a];
    // 1 + q * 2^-15: the byte at mantissa bits 8-15 under 1.0f
    const float Qn = f_of(0x3F800000u | (((wn >> (8 * j)) & 255u) << 8));
    const float Qf = f_of(0x3F800000u | (((wf >> (8 * j)) & 255u) << 8));
    tn[a] = std::fmaf(Qn, A, cn);
    tf[a] = std::fmaf(Qf, A, cf);
  }
  n_out = std::fmax(std::fmax(std::fmax(tn[0], tn[1]), tn[2]), cull_lo);
  f_out = std::fmin(std::fmin(std::fmin(tf[0], tf[1]), tf[2]), cull_hi);
}

void check_scene(const Scene& sc, uint32_t paths) {
  const uint32_t nt = (uint32_t)sc.tris.size();
  std::vector<RtBVHNode40> nodes(2 * (size_t)nt - 1);
  build_sah(sc.tris.data(), nt, nullptr, 0, nodes.data());
  HostDeviceBVH hb;
  std::string msg;
  if (!convert_bvh(nodes.data(), (uint32_t)nodes.size(), sc.tris.data(), nt, nullptr, 0, nullptr, 0, 1, 0, hb, msg)) {
    fail(sc.name + ": convert_bvh: " + msg);
    return;
  }
  if (hb.width != 4) {
    fail(sc.name + ": expected 4-wide nodes");
    return;
  }
  const size_t nn = hb.inner.size() / 16;
  const uint32_t kEmpty = kLeafBit | kSphereBit | kSphereMask;
  // exact primitive bounds of every wide node (filled in post-order below)
  std::vector<Box> nb(nn);
  auto tri_box = [&](uint32_t slot) {
    const RtTriangle64& t = sc.tris[hb.tri_ids[slot]];
    Box b;
    for (const float* v : {t.v0, t.v1, t.v2})
      for (int a = 0; a < 3; ++a) {
        b.lo[a] = std::fmin(b.lo[a], (double)v[a]);
        b.hi[a] = std::fmax(b.hi[a], (double)v[a]);
      }
    return b;
  };
  auto ref_box = [&](uint32_t r) {
    Box b;
    if (r & kLeafBit) {
      const uint32_t first = r & kSlotMask, count = ((r >> kCountShift) & 7u) + 1u;
      for (uint32_t k = 0; k < count; ++k) b.grow(tri_box(first + k));
    } else {
      b = nb[r];
    }
    return b;
  };
  std::vector<int> parent(nn, -1), pslot(nn, -1);
  std::vector<std::pair<uint32_t, int>> leaf_of(hb.tri_ids.size(), {0u, -1});
  for (size_t i = 0; i < nn; ++i)
    for (int j = 0; j < 4; ++j) {
      const uint32_t r = u_of(hb.inner[16 * i + 4 + j]);
      if (r == kEmpty) continue;
      if (r & kLeafBit) {
        const uint32_t first = r & kSlotMask, count = ((r >> kCountShift) & 7u) + 1u;
        for (uint32_t k = 0; k < count; ++k) leaf_of[first + k] = {(uint32_t)i, j};
      } else {
        parent[r] = (int)i;
        pslot[r] = j;
      }
    }
  // post-order over the wide tree from the root
  {
    std::vector<std::pair<uint32_t, bool>> st{{hb.root, false}};
    while (!st.empty()) {
      auto [x, done] = st.back();
      st.pop_back();
      if (done) {
        Box b;
        for (int j = 0; j < 4; ++j) {
          const uint32_t r = u_of(hb.inner[16 * x + 4 + j]);
          if (r != kEmpty) b.grow(ref_box(r));
        }
        nb[x] = b;
        continue;
      }
      st.push_back({x, true});
      for (int j = 0; j < 4; ++j) {
        const uint32_t r = u_of(hb.inner[16 * x + 4 + j]);
        if (r != kEmpty && !(r & kLeafBit)) st.push_back({r, false});
      }
    }
  }
  // encode: exact enclosure
  const int ax_scale[3] = {3, 14, 15};
  for (size_t i = 0; i < nn; ++i) {
    const float* nd = &hb.inner[16 * i];
    for (int j = 0; j < 4; ++j) {
      const uint32_t r = u_of(nd[4 + j]);
      if (r == kEmpty) continue;
      const Box b = ref_box(r);
      for (int a = 0; a < 3; ++a) {
        const double st = (double)nd[ax_scale[a]] / 32768.0;
        const uint32_t ql = (u_of(nd[8 + 2 * a]) >> (8 * j)) & 255u, qh = (u_of(nd[9 + 2 * a]) >> (8 * j)) & 255u;
        // p + ql*st <= lo  and  p + qh*st >= hi
        if (exact_sign({(double)nd[a], (double)ql * st, -b.lo[a]}) > 0 ||
            exact_sign({(double)nd[a], (double)qh * st, -b.hi[a]}) < 0) {
          char buf[256];
          std::snprintf(buf, sizeof buf, "%s: node %zu slot %d axis %d: planes [%u, %u] of p=%.9g step %.9g miss [%.9g, %.9g]",
                        sc.name.c_str(), i, j, a, ql, qh, (double)nd[a], st, b.lo[a], b.hi[a]);
          fail(buf);
        }
      }
    }
  }
  // visit: random rays through random triangles' bounds, every node on the path
  std::mt19937_64 g(12345);
  std::uniform_real_distribution<double> u(0.0, 1.0);
  const Box root = nb[hb.root];
  double span = 0.0;
  for (int a = 0; a < 3; ++a) span = std::fmax(span, root.hi[a] - root.lo[a]);
  if (span == 0.0) span = 1.0;
  for (uint32_t p = 0; p < paths; ++p) {
    const uint32_t slot = (uint32_t)(u(g) * (double)hb.tri_ids.size()) % (uint32_t)hb.tri_ids.size();
    const Box tb = tri_box(slot);
    float o[3], d[3];
    double tgt[3];
    for (int a = 0; a < 3; ++a) {
      tgt[a] = tb.lo[a] + u(g) * (tb.hi[a] - tb.lo[a]);
      o[a] = (float)(root.lo[a] + (u(g) * 1.4 - 0.2) * span);
    }
    const int axis_ray = (int)(u(g) * 4.0);  // 0-2: one direction component exactly 0
    double len = 0.0;
    double dd[3];
    for (int a = 0; a < 3; ++a) {
      dd[a] = tgt[a] - (double)o[a];
      if (a == axis_ray) {
        dd[a] = 0.0;
        o[a] = (float)tgt[a];
      }
      len += dd[a] * dd[a];
    }
    len = std::sqrt(len);
    if (len == 0.0) continue;
    for (int a = 0; a < 3; ++a) d[a] = (float)(dd[a] / len);
    // walk up from the leaf slot
    uint32_t node = leaf_of[slot].first;
    int j = leaf_of[slot].second;
    Box child = ref_box(u_of(hb.inner[16 * node + 4 + j]));
    for (;;) {
      // exact entry/exit of the ray (o + t d, binary64 from the float o, d) in `child`
      double t0 = -INFINITY, t1 = INFINITY;
      bool empty = false;
      for (int a = 0; a < 3; ++a) {
        if (d[a] == 0.0f) {
          if ((double)o[a] < child.lo[a] || (double)o[a] > child.hi[a]) empty = true;
          continue;
        }
        double a0 = (child.lo[a] - (double)o[a]) / (double)d[a], a1 = (child.hi[a] - (double)o[a]) / (double)d[a];
        if (a0 > a1) std::swap(a0, a1);
        t0 = std::fmax(t0, a0);
        t1 = std::fmin(t1, a1);
      }
      if (!empty && t0 <= t1) {
        float n, f;
        visit_child(&hb.inner[16 * node], j, o, d, -INFINITY, INFINITY, n, f);
        // [t0, t1] in binary64 from binary32 inputs: within 1e-12 of exact
        const double tol = 1e-12 * (std::fabs(t0) + std::fabs(t1));
        if (!((double)n <= t0 + tol && t1 - tol <= (double)f)) {
          char buf[256];
          std::snprintf(buf, sizeof buf, "%s: path %u node %u slot %d: box on [%.9g, %.9g], visit gives [%.9g, %.9g]",
                        sc.name.c_str(), p, node, j, t0, t1, (double)n, (double)f);
          fail(buf);
          break;
        }
      }
      if (parent[node] < 0) break;
      j = pslot[node];
      node = (uint32_t)parent[node];
      child = nb[u_of(hb.inner[16 * node + 4 + j])];
    }
  }
  std::printf("ok %s %zu %u\n", sc.name.c_str(), nn, paths);
}

}  // namespace

int main() {
  std::vector<Scene> scenes;
  const double zero[3] = {0, 0, 0};
  scenes.push_back({"unit-soup", soup(1, 20000, 1.0, 0.002, zero)});
  const double far1[3] = {1.0e6, -2.5e7, 3.3e3};
  scenes.push_back({"offset-1e7", soup(2, 20000, 1000.0, 2.0, far1)});
  const double far2[3] = {1.0, 2.0, -3.0};
  scenes.push_back({"tiny-at-1", soup(3, 5000, 1e-6, 2e-9, far2)});
  const double far3[3] = {0.25, -0.5, 0.3};
  scenes.push_back({"flat-z", soup(4, 5000, 1.0, 0.01, far3, true)});
  const double far4[3] = {1.0e17, -3.0e17, 5.0e17};
  scenes.push_back({"huge-1e17", soup(5, 5000, 1.0e15, 1.0e12, far4)});
  const double mid[3] = {-1.0, -1.0, -1.0};
  scenes.push_back({"signed", soup(6, 20000, 2.0, 0.01, mid)});
  scenes.push_back({"subnormal", soup(7, 3000, 1e-40, 1e-43, zero)});
  const double far5[3] = {1.0e9, 1.0e9, -1.0e9};
  scenes.push_back({"wide-1e9", soup(8, 10000, 2.0e9, 1.0e6, far5)});
  for (const Scene& s : scenes) check_scene(s, 4000);

  // wider than 255 * 2^48: the default layout is binary, 4-wide is refused
  const double far6[3] = {2.0e18, 0.0, 0.0};
  std::vector<RtTriangle64> t = soup(9, 1000, 1.0e17, 1.0e14, far6);
  std::vector<RtBVHNode40> nodes(2 * t.size() - 1);
  build_sah(t.data(), (uint32_t)t.size(), nullptr, 0, nodes.data());
  HostDeviceBVH hb;
  std::string msg;
  if (!convert_bvh(nodes.data(), (uint32_t)nodes.size(), t.data(), (uint32_t)t.size(), nullptr, 0, nullptr, 0, 1, 0,
                   hb, msg) || hb.width != 2)
    fail("wide-1e17: expected binary nodes by default");
  if (convert_bvh(nodes.data(), (uint32_t)nodes.size(), t.data(), (uint32_t)t.size(), nullptr, 0, nullptr, 0, 1, 4, hb,
                  msg))
    fail("wide-1e17: 4-wide nodes accepted");
  else
    std::printf("ok wide-1e17 refused: %s\n", msg.c_str());
  return g_fail ? 1 : 0;
}
