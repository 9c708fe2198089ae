// mh_oracle.cpp -- TEST INFRASTRUCTURE ONLY: the CPU oracle of the fusion path.
//
// A scalar C++ restatement of MeshHashing's update rules, used by the tests,
// by __graft_entry__.smoke() and by bench.py's CPU-baseline leg as the checker.
// Nothing in the product (meshhashing_gb300/) links, loads or calls it.
//
// The arithmetic is templated on R:
//   R = double : the FP64 oracle ("truth"); the reference's formulas evaluated
//                in double.
//   R = float  : the FP32-faithful oracle; the same formulas, in the same
//                operation order, in IEEE single precision with no FMA
//                contraction (-ffp-contract=off).  Discrete decisions (DDA
//                block visits, projection rounding, cube indices, validity
//                gates) are made exactly as an FP32 implementation makes them.
//
// Each function cites the reference file:line it follows.  Deliberate,
// documented departures from the reference (all shared with the GPU path):
//   * allocation inserts every touched in-frustum block (the reference drops
//     inserts when two new blocks share a bucket in one frame,
//     core/hash_table.h:133-176);
//   * a shared MC vertex is computed once per frame from its owner cube's
//     view of the edge (the reference lets the last of up to four writers win,
//     meshing/marching_cubes.cu:41-71);
//   * a vertex whose trilinear sample is invalid gets radius 0 (the reference
//     reads an uninitialised local, marching_cubes.cu:50-55);
//   * the low-surfel GC updates all life counters before testing neighbours
//     (the reference relies on __syncthreads across CTAs, recycle.cu:94-113);
//   * deleting a hash entry never fails (the reference's FreeEntry gives up
//     when the bucket mutex is still held, core/hash_table.h:199-244);
//   * FP32 mode uses algebraically equal, well-conditioned forms of the PSDF
//     update (update_bayesian.cu:140-181: the variance without its
//     cancellation, the Beta moments over one denominator, 4 divisions in
//     all); FP64 mode uses the reference's form.
#include <algorithm>
#include <atomic>
#include <cassert>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <memory>
#include <unordered_map>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/meshhash.h"
#include "../meshhashing_gb300/csrc/mh_exp.h"

namespace orc {

static const int kB = 8;          // BLOCK_SIDE_LENGTH (core/common.h:48)
static const int kBV = 512;       // BLOCK_SIZE
static const int kBlockLife = 3;  // BLOCK_LIFE (core/block.h:13)

// float -> int conversion with round-toward-zero and the saturating NaN -> 0
// behaviour of the GPU's cvt.rzi.s32.f32, so both sides agree on every input.
template <class R> static inline int f2i(R v) {
  if (v != v) return 0;
  if (v >= (R)2147483647.0) return INT_MAX;
  if (v <= (R)-2147483648.0) return INT_MIN;
  return (int)v;
}

template <class R> struct V3 {
  R x, y, z;
};
template <class R> static inline V3<R> mk(R x, R y, R z) { return V3<R>{x, y, z}; }
template <class R> static inline V3<R> operator+(V3<R> a, V3<R> b) { return mk(a.x + b.x, a.y + b.y, a.z + b.z); }
template <class R> static inline V3<R> operator-(V3<R> a, V3<R> b) { return mk(a.x - b.x, a.y - b.y, a.z - b.z); }
template <class R> static inline V3<R> operator*(V3<R> a, R s) { return mk(a.x * s, a.y * s, a.z * s); }
template <class R> static inline V3<R> operator*(R s, V3<R> a) { return mk(s * a.x, s * a.y, s * a.z); }
template <class R> static inline V3<R> operator/(V3<R> a, R s) { return mk(a.x / s, a.y / s, a.z / s); }
template <class R> static inline R dot(V3<R> a, V3<R> b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
// normalize = v * (1 / sqrt(v.v)); the host form of helper_math's normalize.
template <class R> static inline V3<R> normalize(V3<R> v) {
  R inv = (R)1 / std::sqrt(dot(v, v));
  return v * inv;
}
template <class R> static inline R length(V3<R> v) { return std::sqrt(dot(v, v)); }

struct I3 {
  int x, y, z;
};
static inline bool operator==(I3 a, I3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }

// Row-major 4x4 (extern/cuda/matrix.h float4x4).
template <class R> struct M4 {
  R e[16];
  // point transform, w = 1 (matrix.h:920-926)
  V3<R> pt(V3<R> v) const {
    return mk(e[0] * v.x + e[1] * v.y + e[2] * v.z + e[3] * (R)1,
              e[4] * v.x + e[5] * v.y + e[6] * v.z + e[7] * (R)1,
              e[8] * v.x + e[9] * v.y + e[10] * v.z + e[11] * (R)1);
  }
  // direction transform, w = 0 (matrix.h:908-916, xyz part)
  V3<R> dir(V3<R> v) const {
    return mk(e[0] * v.x + e[1] * v.y + e[2] * v.z + e[3] * (R)0,
              e[4] * v.x + e[5] * v.y + e[6] * v.z + e[7] * (R)0,
              e[8] * v.x + e[9] * v.y + e[10] * v.z + e[11] * (R)0);
  }
};

// General 4x4 inverse by cofactors, with the term order of
// float4x4::getInverse (extern/cuda/matrix.h:964-1086): each cofactor is the
// 3x3 minor expanded along its first remaining column, terms summed left to
// right, then scaled by 1/det.
template <class R> static M4<R> inverse(const M4<R> &m) {
  R inv[16];
  for (int r = 0; r < 4; ++r) {
    for (int c = 0; c < 4; ++c) {
      // inverse entry (r, c) = cofactor of original (c, r) / det
      int rows[3], cols[3], nr = 0, nc = 0;
      for (int i = 0; i < 4; ++i) if (i != c) rows[nr++] = i;
      for (int j = 0; j < 4; ++j) if (j != r) cols[nc++] = j;
      auto E = [&](int i, int j) { return m.e[i * 4 + j]; };
      int ra = rows[0], rb = rows[1], rc = rows[2];
      int c0 = cols[0], c1 = cols[1], c2 = cols[2];
      R s = ((r + c) & 1) ? (R)-1 : (R)1;
      R t[6];
      t[0] = (s * E(ra, c0)) * E(rb, c1) * E(rc, c2);
      t[1] = -((s * E(ra, c0)) * E(rb, c2) * E(rc, c1));
      t[2] = -((s * E(rb, c0)) * E(ra, c1) * E(rc, c2));
      t[3] = (s * E(rb, c0)) * E(ra, c2) * E(rc, c1);
      t[4] = (s * E(rc, c0)) * E(ra, c1) * E(rb, c2);
      t[5] = -((s * E(rc, c0)) * E(ra, c2) * E(rb, c1));
      R acc = t[0];
      for (int k = 1; k < 6; ++k) acc = acc + t[k];
      inv[r * 4 + c] = acc;
    }
  }
  R det = m.e[0] * inv[0] + m.e[1] * inv[4] + m.e[2] * inv[8] + m.e[3] * inv[12];
  R detr = (R)1 / det;
  M4<R> out;
  for (int i = 0; i < 16; ++i) out.e[i] = inv[i] * detr;
  return out;
}

// ---------------------------------------------------------------- hashing

// Teschner spatial hash with int32 wrap-around and unsigned modulo
// (core/hash_table.h:259-269).
static inline uint32_t hash_bucket(int x, int y, int z, uint32_t bucket_count) {
  uint32_t h = ((uint32_t)x * 73856093u) ^ ((uint32_t)y * 19349669u) ^ ((uint32_t)z * 83492791u);
  return h % bucket_count;
}

static inline uint64_t bkey(int x, int y, int z) {
  const uint64_t M = 0x1FFFFF;
  return (((uint64_t)x & M) << 42) | (((uint64_t)y & M) << 21) | ((uint64_t)z & M);
}
static inline int sext21(uint64_t v) { return (int)((int64_t)(v << 43) >> 43); }
static inline I3 unkey(uint64_t k) { return I3{sext21(k >> 42), sext21(k >> 21), sext21(k)}; }

// vertex key: owner voxel (20-bit signed coords) and slot
static inline uint64_t vkey(int x, int y, int z, int slot) {
  const uint64_t M = 0xFFFFF;
  return (((uint64_t)x & M) << 42) | (((uint64_t)y & M) << 22) | (((uint64_t)z & M) << 2) | (uint64_t)slot;
}
static inline int sext20(uint64_t v) { return (int)((int64_t)(v << 44) >> 44); }

// ---------------------------------------------------------------- MC tables
// Bourke's public triangle table (meshing/mc_tables.h:10-14 cites the same
// source), packed one uint64 per case; the edge mask of a case is derived
// from the corner signs instead of being stored.
#define MH_MC_TABLE_QUALIFIER static const
#include "../meshhashing_gb300/csrc/mc_cases.inc"
static inline int case_edge(int c, int k) { return (int)((kMcCases[c] >> (4 + 4 * k)) & 0xF); }

// Reference cube-corner numbering (meshing/mc_tables.h:335-344): corner i sits
// at voxel offset kVtx[i]; edge e joins corners kEdgeEnds[e]; the vertex of
// edge e is owned by the cube at offset kOwner[e].xyz, slot kOwner[e].w
// (mc_tables.h:360-390).
static const int kVtx[8][3] = {{0, 1, 1}, {1, 1, 1}, {1, 1, 0}, {0, 1, 0},
                               {0, 0, 1}, {1, 0, 1}, {1, 0, 0}, {0, 0, 0}};
static const int kEdgeEnds[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                     {6, 7}, {7, 4}, {4, 0}, {5, 1}, {6, 2}, {7, 3}};
static int kOwner[12][4];  // derived in init_tables()
static int kCaseEdges[256];
static bool tables_ready = false;

static void init_tables() {
  if (tables_ready) return;
  for (int e = 0; e < 12; ++e) {
    const int *p = kVtx[kEdgeEnds[e][0]], *q = kVtx[kEdgeEnds[e][1]];
    int axis = p[0] != q[0] ? 0 : (p[1] != q[1] ? 1 : 2);
    int lo[3] = {std::min(p[0], q[0]), std::min(p[1], q[1]), std::min(p[2], q[2])};
    kOwner[e][0] = lo[0];
    kOwner[e][1] = lo[1];
    kOwner[e][2] = lo[2];
    kOwner[e][3] = axis;
  }
  for (int c = 0; c < 256; ++c) {
    int m = 0;
    for (int e = 0; e < 12; ++e) {
      int a = (c >> kEdgeEnds[e][0]) & 1, b = (c >> kEdgeEnds[e][1]) & 1;
      if (a != b) m |= 1 << e;
    }
    kCaseEdges[c] = m;
  }
  tables_ready = true;
}
static inline int case_tri_count(int c) { return (int)(kMcCases[c] & 0xF); }

// ---------------------------------------------------------------- state

template <class R> struct Blk {
  int x, y, z;
  R sdf[kBV], w[kBV], a[kBV], b[kBV];
  int life = kBlockLife, inner = 0, boundary = 0;
  uint8_t cube[kBV];
  uint8_t flag = 0;
  Blk() {
    for (int i = 0; i < kBV; ++i) sdf[i] = w[i] = a[i] = b[i] = 0;
    memset(cube, 0, sizeof(cube));
  }
};

template <class R> struct Vtx {
  R pos[3] = {0, 0, 0}, normal[3] = {0, 0, 0}, radius = 0;
  int ref = 0;
  uint32_t epoch = 0;
};
struct Tris {
  uint8_t n = 0;
  uint64_t v[5][3];
};

template <class R> struct Vol {
  mh_params p;
  std::vector<std::unique_ptr<Blk<R>>> blocks;  // may contain nulls after GC
  std::unordered_map<uint64_t, int> index;
  std::vector<int> cand;                        // candidate block indices
  std::vector<uint64_t> touched;                // blocks met by the last allocation
  std::unordered_map<uint64_t, Vtx<R>> verts;
  std::unordered_map<uint64_t, Tris> tris;      // key: vkey(cube voxel, 0)
  uint32_t epoch = 0;
  int frames = 0;
  // current frame
  std::vector<float> depth;   // preprocessed
  std::vector<float> inlier;
  M4<R> wTc, cTw;
  M4<float> cTw_f;

  int find(int x, int y, int z) const {
    auto it = index.find(bkey(x, y, z));
    return it == index.end() ? -1 : it->second;
  }
  int insert(int x, int y, int z) {
    uint64_t k = bkey(x, y, z);
    auto it = index.find(k);
    if (it != index.end()) return it->second;
    auto b = std::make_unique<Blk<R>>();
    b->x = x, b->y = y, b->z = z;
    int id = (int)blocks.size();
    blocks.push_back(std::move(b));
    index[k] = id;
    return id;
  }
  void erase(int id) {
    Blk<R> *b = blocks[id].get();
    index.erase(bkey(b->x, b->y, b->z));
    blocks[id].reset();
  }

  // ---------------------------------------------------------- geometry
  // geometry/geometry_helper.h:36-216
  R vs() const { return (R)p.voxel_size; }
  V3<R> world_to_voxelf(V3<R> w) const { return w / vs(); }
  I3 world_to_voxeli(V3<R> w) const {
    V3<R> q = w / vs();
    auto rnd = [](R v) { R s = v < (R)0 ? (R)-1 : (R)1; return f2i<R>(v + s * (R)0.5); };
    return I3{rnd(q.x), rnd(q.y), rnd(q.z)};
  }
  V3<R> voxel_to_world(I3 v) const { return mk((R)v.x, (R)v.y, (R)v.z) * vs(); }
  static I3 voxel_to_block(I3 v) {
    return I3{(v.x - (v.x < 0) * (kB - 1)) / kB, (v.y - (v.y < 0) * (kB - 1)) / kB,
              (v.z - (v.z < 0) * (kB - 1)) / kB};
  }
  static I3 block_to_voxel(I3 b) { return I3{b.x * kB, b.y * kB, b.z * kB}; }
  I3 world_to_block(V3<R> w) const { return voxel_to_block(world_to_voxeli(w)); }
  V3<R> block_to_world(I3 b) const { return voxel_to_world(block_to_voxel(b)); }
  R truncate(R z) const { return (R)p.truncation_distance + (R)p.truncation_distance_scale * z; }
  R normalize_depth(R z) const {
    return (z - (R)p.min_depth_range) / ((R)p.max_depth_range - (R)p.min_depth_range);
  }
  void project_f(V3<R> c, R fx, R fy, R cx, R cy, R &u, R &v) const {
    u = c.x * fx / c.z + cx;
    v = c.y * fy / c.z + cy;
  }
  void project_i(V3<R> c, int &u, int &v) const {
    R uf, vf;
    project_f(c, (R)p.fx, (R)p.fy, (R)p.cx, (R)p.cy, uf, vf);
    u = f2i<R>(uf + (R)0.5);
    v = f2i<R>(vf + (R)0.5);
  }
  V3<R> reproject(unsigned ux, unsigned uy, R d, R fx, R fy, R cx, R cy) const {
    R x = ((R)ux - cx) / fx;
    R y = ((R)uy - cy) / fy;
    return mk(d * x, d * y, d);
  }
  bool point_in_frustum(const M4<R> &cTw_, V3<R> w) const {
    V3<R> c = cTw_.pt(w);
    R u, v;
    project_f(c, (R)p.fx, (R)p.fy, (R)p.cx, (R)p.cy, u, v);
    R W1 = (R)p.width - (R)1, H1 = (R)p.height - (R)1;
    V3<R> n = mk(((R)2 * u - W1) / W1, (H1 - (R)2 * v) / H1, normalize_depth(c.z));
    R s = (R)0.95f;
    if (sizeof(R) == 8) s = (R)0.95;
    n = n * s;
    const R one = 1, zero = 0;
    return !((n.x < -one) || (n.x > one) || (n.y < -one) || (n.y > one) || (n.z < zero) || (n.z > one));
  }
  bool block_in_frustum(const M4<R> &cTw_, I3 b) const {
    V3<R> w = block_to_world(b);
    R off = vs() * (R)0.5 * ((R)kB - (R)1);
    return point_in_frustum(cTw_, mk(w.x + off, w.y + off, w.z + off));
  }

  // ---------------------------------------------------------- frame input
  // Sensor::Process (sensor/rgbd_sensor.cu:118-137, preprocess.cu:10-42)
  void frame_set(const float *d, const float *wtc) {
    size_t n = (size_t)p.width * p.height;
    depth.resize(n);
    inlier.assign(n, 0.1f);
    for (size_t i = 0; i < n; ++i) {
      float z = d[i];
      bool ok = z >= p.min_depth_range && z <= p.max_depth_range;
      depth[i] = ok ? z : -INFINITY;
    }
    M4<float> wf;
    for (int i = 0; i < 16; ++i) wf.e[i] = wtc[i];
    M4<float> cf = inverse(wf);
    cTw_f = cf;
    for (int i = 0; i < 16; ++i) {
      wTc.e[i] = (R)wf.e[i];
    }
    // FP32 mode uses the float inverse bit for bit; FP64 inverts in double.
    cTw = sizeof(R) == 4 ? M4<R>{} : inverse(wTc);
    if (sizeof(R) == 4)
      for (int i = 0; i < 16; ++i) cTw.e[i] = (R)cf.e[i];
  }
  // Chambolle-Pock TV-L2 on the depth frame in millimetres (no reference
  // counterpart; the same method as the library's denoiser, evaluated in
  // double): forward differences over valid pixel pairs, tau = sigma =
  // 1/sqrt(8), theta = 1, invalid pixels stay invalid.
  void denoise_tv(double lambda, int iters) {
    if (sizeof(R) == 4) {
      denoise_tv_f32((float)lambda, iters);
      return;
    }
    const int W = p.width, H = p.height;
    const size_t n = (size_t)W * H;
    std::vector<double> f(n, 0), u(n), ub(n), px(n, 0), py(n, 0), u2(n), ub2(n), px2(n), py2(n);
    std::vector<uint8_t> ok(n);
    for (size_t i = 0; i < n; ++i) {
      float z = depth[i];
      ok[i] = z > 0.0f && z < 1e30f;
      f[i] = ok[i] ? (double)z * 1000.0 : 0.0;
      u[i] = ub[i] = f[i];
    }
    const double tau = 1.0 / std::sqrt(8.0), sigma = tau;
    auto dual = [&](int x, int y, double &ox, double &oy) {
      size_t i = (size_t)y * W + x;
      double gx = 0, gy = 0;
      if (ok[i] && x + 1 < W && ok[i + 1]) gx = ub[i + 1] - ub[i];
      if (ok[i] && y + 1 < H && ok[i + W]) gy = ub[i + W] - ub[i];
      double qx = px[i] + sigma * gx, qy = py[i] + sigma * gy;
      double nr = std::max(1.0, std::sqrt(qx * qx + qy * qy));
      ox = qx / nr, oy = qy / nr;
    };
    for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
      for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
          size_t i = (size_t)y * W + x;
          double pxc, pyc, pxl = 0, pyu = 0, dm;
          dual(x, y, pxc, pyc);
          px2[i] = pxc, py2[i] = pyc;
          if (!ok[i]) {
            u2[i] = ub2[i] = f[i];
            continue;
          }
          if (x > 0) dual(x - 1, y, pxl, dm);
          if (y > 0) dual(x, y - 1, dm, pyu);
          double div = (pxc - pxl) + (pyc - pyu);
          double un = (u[i] + tau * div + tau * lambda * f[i]) / (1.0 + tau * lambda);
          u2[i] = un;
          ub2[i] = 2.0 * un - u[i];
        }
      }
      u.swap(u2), ub.swap(ub2), px.swap(px2), py.swap(py2);
    }
    for (size_t i = 0; i < n; ++i) depth[i] = ok[i] ? (float)(u[i] * 0.001) : -INFINITY;
  }

  // The same iteration in single precision, in the operation order of the
  // library's kernels (every value a correctly rounded +, -, *, /, sqrt or
  // max of the previous iterate), so its output is bit-identical to theirs:
  // depth in millimetres z * 1000, tau = sigma = 1/sqrt(8) rounded to float,
  // u' = (u + tau div + (tau lambda) f) / (1 + tau lambda), output u' * 0.001.
  void denoise_tv_f32(float lambda, int iters) {
    const int W = p.width, H = p.height;
    const size_t n = (size_t)W * H;
    std::vector<float> f(n), u(n), ub(n), px(n, 0.0f), py(n, 0.0f), u2(n), ub2(n), px2(n), py2(n);
    std::vector<uint8_t> ok(n);
    for (size_t i = 0; i < n; ++i) {
      const float z = depth[i];
      ok[i] = z > 0.0f && z < 1e30f;
      f[i] = ok[i] ? z * 1000.0f : -INFINITY;
      u[i] = ub[i] = f[i];
    }
    const float tau = 0.35355339059327373f, sigma = 0.35355339059327373f;
    auto dual = [&](int x, int y, float &ox, float &oy) {
      const size_t i = (size_t)y * W + x;
      float gx = 0.0f, gy = 0.0f;
      if (ok[i] && x + 1 < W && ok[i + 1]) gx = ub[i + 1] - ub[i];
      if (ok[i] && y + 1 < H && ok[i + W]) gy = ub[i + W] - ub[i];
      const float qx = px[i] + sigma * gx, qy = py[i] + sigma * gy;
      const float nr = std::fmax(1.0f, std::sqrt(qx * qx + qy * qy));
      ox = qx / nr, oy = qy / nr;
    };
    for (int it = 0; it < iters; ++it) {
#pragma omp parallel for schedule(static)
      for (int y = 0; y < H; ++y) {
        for (int x = 0; x < W; ++x) {
          const size_t i = (size_t)y * W + x;
          float pxc, pyc, pxl = 0.0f, pyu = 0.0f, dm;
          dual(x, y, pxc, pyc);
          px2[i] = pxc, py2[i] = pyc;
          if (!ok[i]) {
            u2[i] = ub2[i] = f[i];
            continue;
          }
          if (x > 0) dual(x - 1, y, pxl, dm);
          if (y > 0) dual(x, y - 1, dm, pyu);
          const float div = (pxc - pxl) + (pyc - pyu);
          const float u0 = u[i];
          const float un = (u0 + tau * div + tau * lambda * f[i]) / (1.0f + tau * lambda);
          u2[i] = un;
          ub2[i] = 2.0f * un - u0;
        }
      }
      u.swap(u2), ub.swap(ub2), px.swap(px2), py.swap(py2);
    }
    for (size_t i = 0; i < n; ++i) depth[i] = ok[i] ? u[i] * 0.001f : -INFINITY;
  }

  bool depth_invalid(float d) const {
    return d == -INFINITY || d == 0.0f || d >= p.sdf_upper_bound;
  }

  // ---------------------------------------------------------- allocation
  // AllocBlockArrayKernel (mapping/allocate.cu:8-99): per-pixel DDA over the
  // blocks met by [d - mu(d), d + mu(d)], inserting every in-frustum block.
  void alloc_pixel(unsigned x, unsigned y, std::vector<uint64_t> &out) const {
    float df = depth[(size_t)y * p.width + x];
    if (depth_invalid(df)) return;
    R d = (R)df;
    R ub = (R)p.sdf_upper_bound;
    R tr = truncate(d);
    R near_d = std::min(ub, d - tr);
    R far_d = std::min(ub, d + tr);
    if (near_d >= far_d) return;
    V3<R> cn = reproject(x, y, near_d, (R)p.fx, (R)p.fy, (R)p.cx, (R)p.cy);
    V3<R> cf = reproject(x, y, far_d, (R)p.fx, (R)p.fy, (R)p.cx, (R)p.cy);
    V3<R> wn = wTc.pt(cn), wf = wTc.pt(cf);
    V3<R> dir = normalize(wf - wn);
    I3 bn = world_to_block(wn), bf = world_to_block(wf);
    V3<R> st = mk(dir.x < 0 ? (R)-1 : (R)1, dir.y < 0 ? (R)-1 : (R)1, dir.z < 0 ? (R)-1 : (R)1);
    I3 bo{bn.x + (st.x > 0 ? 1 : 0), bn.y + (st.y > 0 ? 1 : 0), bn.z + (st.z > 0 ? 1 : 0)};
    V3<R> bw = block_to_world(bo);
    R hv = (R)0.5 * vs();
    V3<R> cen = mk(bw.x - hv, bw.y - hv, bw.z - hv);
    V3<R> t = mk((cen.x - wn.x) / dir.x, (cen.y - wn.y) / dir.y, (cen.z - wn.z) / dir.z);
    V3<R> s8 = st * (R)kB;
    V3<R> dt = mk(s8.x * vs() / dir.x, s8.y * vs() / dir.y, s8.z * vs() / dir.z);
    I3 bound{f2i<R>((R)bf.x + st.x), f2i<R>((R)bf.y + st.y), f2i<R>((R)bf.z + st.z)};
    const R inf = (R)INFINITY;
    if (dir.x == (R)0) t.x = dt.x = inf;
    if (dir.y == (R)0) t.y = dt.y = inf;
    if (dir.z == (R)0) t.z = dt.z = inf;
    I3 cur = bn;
    for (int it = 0; it < 1024; ++it) {
      if (block_in_frustum(cTw, cur)) out.push_back(bkey(cur.x, cur.y, cur.z));
      if (t.x < t.y && t.x < t.z) {
        cur.x = f2i<R>((R)cur.x + st.x);
        if (cur.x == bound.x) return;
        t.x += dt.x;
      } else if (t.y < t.z) {
        cur.y = f2i<R>((R)cur.y + st.y);
        if (cur.y == bound.y) return;
        t.y += dt.y;
      } else {
        cur.z = f2i<R>((R)cur.z + st.z);
        if (cur.z == bound.z) return;
        t.z += dt.z;
      }
    }
  }
  // returns the set of touched blocks (sorted keys); inserts new ones
  std::vector<uint64_t> allocate() {
    int W = p.width, H = p.height;
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    std::vector<std::vector<uint64_t>> per(nt);
#pragma omp parallel for schedule(dynamic, 4)
    for (int y = 0; y < H; ++y) {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      for (int x = 0; x < W; ++x) alloc_pixel(x, y, per[tid]);
    }
    std::vector<uint64_t> all;
    for (auto &v : per) all.insert(all.end(), v.begin(), v.end());
    std::sort(all.begin(), all.end());
    all.erase(std::unique(all.begin(), all.end()), all.end());
    for (uint64_t k : all) {
      I3 b = unkey(k);
      insert(b.x, b.y, b.z);
    }
    touched = all;
    return all;
  }

  // ---------------------------------------------------------- collect
  // CollectBlocksInFrustumKernel (core/collect_block_array.cu:25-59)
  void collect_frustum() {
    cand.clear();
    for (int i = 0; i < (int)blocks.size(); ++i) {
      Blk<R> *b = blocks[i].get();
      if (b && block_in_frustum(cTw, I3{b->x, b->y, b->z})) cand.push_back(i);
    }
  }
  void collect_all() {
    cand.clear();
    for (int i = 0; i < (int)blocks.size(); ++i)
      if (blocks[i]) cand.push_back(i);
  }

  // per-voxel projection shared by the update kernels
  // (update_simple.cu:26-46, update_bayesian.cu:154-177, :222-243).  The pixel
  // choice is a discrete decision and is always made in single precision, as
  // the reference makes it; the camera-space depth is computed in R.
  bool project_voxel(const Blk<R> *b, int i, R &cam_z, unsigned &px, unsigned &py, float &dd,
                     float *cam_z_f = nullptr) const {
    I3 vp{b->x * kB + (i % kB), b->y * kB + (i % (kB * kB)) / kB, b->z * kB + i / (kB * kB)};
    const float vsf = p.voxel_size;
    V3<float> wpf = mk((float)vp.x * vsf, (float)vp.y * vsf, (float)vp.z * vsf);
    V3<float> cpf = cTw_f.pt(wpf);
    float uf = cpf.x * p.fx / cpf.z + p.cx;
    float vf = cpf.y * p.fy / cpf.z + p.cy;
    px = (unsigned)f2i<float>(uf + 0.5f), py = (unsigned)f2i<float>(vf + 0.5f);
    if (px >= p.width || py >= p.height) return false;
    dd = depth[(size_t)py * p.width + px];
    if (depth_invalid(dd)) return false;
    cam_z = sizeof(R) == 4 ? (R)cpf.z : cTw.pt(voxel_to_world(vp)).z;
    if (cam_z_f) *cam_z_f = cpf.z;
    return true;
  }

  // the truncation test `sdf <= -mu` (update_simple.cu:57-58) is a discrete
  // decision, made in single precision in both oracle modes
  bool trunc_reject(float d, float cam_z) const {
    float sdf = d - cam_z;
    float tr = p.truncation_distance + p.truncation_distance_scale * d;
    return sdf <= -tr;
  }

  // ---------------------------------------------------------- simple update
  // UpdateBlocksSimpleKernel (mapping/update_simple.cu:13-77), Voxel::Update
  // (core/voxel.h:107-115)
  void integrate_simple() {
#pragma omp parallel for schedule(dynamic, 8)
    for (int ci = 0; ci < (int)cand.size(); ++ci) {
      Blk<R> *b = blocks[cand[ci]].get();
      for (int i = 0; i < kBV; ++i) {
        R cz;
        unsigned px, py;
        float df, czf;
        if (!project_voxel(b, i, cz, px, py, df, &czf)) continue;
        R d = (R)df;
        R sdf = d - cz;
        // update_simple.cu:49-55: w = max(10 ws (1 - normalized depth), 1).  FP32
        // mode evaluates 1 - nd as (dmax - d) / (dmax - dmin), which is exact in
        // the subtraction near the far limit where 1 - nd cancels.
        R w;
        if (sizeof(R) == 8 || p.compat_arithmetic) {
          R nd = normalize_depth(d);
          w = std::max((R)10 * (R)p.weight_sample * ((R)1 - nd), (R)1);
        } else {
          R far = ((R)p.max_depth_range - d) / ((R)p.max_depth_range - (R)p.min_depth_range);
          w = std::max((R)10 * (R)p.weight_sample * far, (R)1);
        }
        R tr = truncate(d);
        if (trunc_reject(df, czf)) continue;
        sdf = sdf >= (R)0 ? std::min(tr, sdf) : std::max(-tr, sdf);
        R W = b->w[i];
        b->sdf[i] = (b->sdf[i] * W + sdf * w) / (W + w);
        b->w[i] = W + w;
      }
    }
  }

  // ---------------------------------------------------------- PSDF
  // exp of the single-precision path: the library's exp (mh_exp.h, basic IEEE
  // operations only, so bit-identical on the GPU and here); the reference's
  // arithmetic (compat) and the FP64 oracle use the C library's
  R ex(R v) const {
    if (sizeof(R) == 4 && !p.compat_arithmetic) return (R)mh_expf((float)v);
    return std::exp(v);
  }
  static R gaussian(R x, R u, R s2) {
    // geometry/geometry_helper.h:30-34 (no 1/2 in the exponent)
    R c = sizeof(R) == 8 ? (R)std::sqrt(2 * M_PI) : (R)2.50662827463100050f;
    return (R)1 / (c * std::sqrt(s2)) * std::exp(-((x - u) * (x - u)) / s2);
  }
  // PredictOutlierRatioKernel (mapping/update_bayesian.cu:36-101); vertices of
  // this voxel's three owner slots drive a per-pixel max of the inlier ratio.
  void predict_inlier() {
    std::vector<std::atomic<uint32_t>> acc(inlier.size());
    for (size_t i = 0; i < inlier.size(); ++i) {
      float v = inlier[i];
      uint32_t u;
      memcpy(&u, &v, 4);
      acc[i].store(u);
    }
#pragma omp parallel for schedule(dynamic, 8)
    for (int ci = 0; ci < (int)cand.size(); ++ci) {
      Blk<R> *b = blocks[cand[ci]].get();
      for (int i = 0; i < kBV; ++i) {
        R cz;
        unsigned px, py;
        float df;
        if (!project_voxel(b, i, cz, px, py, df)) continue;
        int vx = b->x * kB + (i % kB), vy = b->y * kB + (i % (kB * kB)) / kB, vz = b->z * kB + i / (kB * kB);
        V3<R> pc = reproject(px, py, (R)df, (R)p.fx, (R)p.fy, (R)p.cx, (R)p.cy);
        for (int s = 0; s < 3; ++s) {
          auto it = verts.find(vkey(vx, vy, vz, s));
          if (it == verts.end()) continue;
          const Vtx<R> &vt = it->second;
          V3<R> n = mk(vt.normal[0], vt.normal[1], vt.normal[2]);
          V3<R> x = mk(vt.pos[0], vt.pos[1], vt.pos[2]);
          R r = vt.radius;
          // the normal is transformed as a point (with translation), as in
          // update_bayesian.cu:83-86
          V3<R> cn = normalize(cTw.pt(n));
          R cos_a = dot(normalize(mk(-pc.x, -pc.y, -pc.z)), cn);
          V3<R> vec = pc - cTw.pt(x);
          R pd = dot(vec, cn);
          R disk = std::sqrt(dot(vec, vec) - pd * pd);
          R q = pd - b->sdf[i];
          R w_dist = ex(-(q * q) * b->w[i]);
          R w_disk = (R)0.5 + (R)0.5 / ((R)1 + ex(-std::fabs(disk / r)));
          R w_ang = (cos_a - (R)0.1736f) / ((R)1 - (R)0.1736f);
          w_ang = std::fmax(w_ang, (R)0.1f);
          R ir = w_disk * w_dist * w_ang;
          ir = std::fmax(ir, (R)0.01f);
          float irf = (float)ir;
          uint32_t u;
          memcpy(&u, &irf, 4);
          std::atomic<uint32_t> &a = acc[(size_t)py * p.width + px];
          uint32_t old = a.load();
          while (old < u && !a.compare_exchange_weak(old, u)) {
          }
        }
      }
    }
    for (size_t i = 0; i < inlier.size(); ++i) {
      uint32_t u = acc[i].load();
      memcpy(&inlier[i], &u, 4);
    }
  }
  // UpdateBlocksBayesianKernel (mapping/update_bayesian.cu:103-185)
  void integrate_psdf() {
#pragma omp parallel for schedule(dynamic, 8)
    for (int ci = 0; ci < (int)cand.size(); ++ci) {
      Blk<R> *b = blocks[cand[ci]].get();
      for (int i = 0; i < kBV; ++i) {
        R cz;
        unsigned px, py;
        float df, czf;
        if (!project_voxel(b, i, cz, px, py, df, &czf)) continue;
        R d = (R)df;
        R x = d - cz;
        R rho = (R)inlier[(size_t)py * p.width + px];
        R tr = truncate(d);
        if (trunc_reject(df, czf)) continue;
        x = x >= (R)0 ? std::min(tr, x) : std::max(-tr, x);
        R tau = (d - (R)0.4f) * (R)0.012f + (R)0.019f;
        if (b->w[i] == (R)0) {
          b->sdf[i] = x;
          b->w[i] = (R)1 / (tau * tau);
          b->a[i] = rho * (R)10;
          b->b[i] = ((R)1 - rho) * (R)10;
          continue;
        }
        R mu = b->sdf[i];
        R a = b->a[i], bb = b->b[i];
        R t2 = tau * tau;
        const bool in_range = d < (R)p.max_depth_range && d >= (R)p.min_depth_range;
        if (sizeof(R) == 4 && !p.compat_arithmetic) {
          // the single-precision form of the library, same operation order:
          // 4 divisions, with u = w0 sigma^2 and q = 1 / (1 + u) the product's
          // variance is sigma^2 q and its mean q (mu u + x); c = C1 / (C1 + C2);
          // sdf' = mu + c (m - mu); w' = w0 / (c u q + (1 - c) + c (1 - c)(m - mu)^2 w0);
          // a' = (a + c) k, b' = (b + 1 - c) k with
          // k = (c (a - b) - a (b + 1)) / (c^2 (a + b + 2) - (a + 2c)(b + 1)),
          // the reference's Beta moments f (e - f) / (f^2 - e) and a' (1 - f) / f
          // put over one denominator
          const float w0 = (float)b->w[i], muf = (float)mu, xf = (float)x, rf = (float)rho, t2f = (float)t2;
          const float af = (float)a, bf = (float)bb;
          const float u = w0 * t2f;
          const float q = 1.0f / (1.0f + u);
          const float m = q * (muf * u + xf);
          const float isv = w0 * q;
          const float dx = xf - muf;
          const float g = mh_expf(-(dx * dx) * isv) * std::sqrt(isv) * 0.398942280401432678f;
          const float C1 = rf * g;
          const float C2 = in_range ? (1.0f - rf) * 0.204081632653061224f : 1.0f;
          const float c = C1 / (C1 + C2);
          const float oc = 1.0f - c;
          const float dm = m - muf;
          b->sdf[i] = muf + c * dm;
          b->w[i] = w0 / (c * u * q + oc + c * oc * (dm * dm) * w0);
          const float b1 = bf + 1.0f;
          const float kk = (c * (af - bf) - af * b1) / (c * c * (af + bf + 2.0f) - (af + 2.0f * c) * b1);
          b->a[i] = (af + c) * kk;
          b->b[i] = (b1 - c) * kk;
          continue;
        }
        // the reference's expressions (update_bayesian.cu:140-180): in double
        // for the FP64 oracle, in float with its double gaussian() in compat
        R s2 = (R)1 / b->w[i];
        R ss2 = (R)1 / ((R)1 / s2 + (R)1 / t2);
        R m = ss2 * (mu / s2 + x / t2);
        R C1;
        if (sizeof(R) == 4) {
          // the reference's promotion: sqrt(2 pi) is a double (geometry_helper.h:30-34)
          const float sv = (float)(s2 + t2);
          const double g = 1.0 / (2.5066282746310002 * (double)std::sqrt(sv)) *
                           (double)std::exp(-(((float)x - (float)mu) * ((float)x - (float)mu)) / sv);
          C1 = (R)((double)rho * g);
        } else {
          C1 = rho * gaussian(x, mu, s2 + t2);
        }
        R C2 = in_range ? ((R)1 - rho) * (R)1 / ((R)5 - (R)0.1f) : (R)1;
        R sum = C1 + C2;
        C1 /= sum;
        C2 /= sum;
        R f = C1 * (a + 1) / (a + bb + 1) + C2 * a / (a + bb + 1);
        R e = C1 * (a + 1) * (a + 2) / ((a + bb + 1) * (a + bb + 2)) + C2 * a * (a + 1) / ((a + bb + 1) * (a + bb + 2));
        R nsdf = C1 * m + C2 * mu;
        R var = C1 * (ss2 + m * m) + C2 * (s2 + mu * mu) - nsdf * nsdf;
        b->sdf[i] = nsdf;
        b->w[i] = (R)1 / var;
        R na = (e - f) / (f - e / f);
        b->a[i] = na;
        b->b[i] = na * ((R)1 - f) / f;
      }
    }
  }

  // ---------------------------------------------------------- Huber-TV
  // Primal-dual state of PrimalDualVariables (core/voxel.h:62-82), kept for
  // the blocks that were candidates at the last init; other blocks read as
  // unmasked.
  struct PDB {
    R sdf0[kBV], bar[kBV], w[kBV], p[kBV][3];
    bool mask[kBV];
  };
  std::unordered_map<int, std::unique_ptr<PDB>> pd;
  double pd_err[2] = {0, 0};

  // block id and local index of voxel v, -1 when its block does not exist
  int voxel_id(I3 v, int &li) const {
    I3 bp = voxel_to_block(v);
    int id = find(bp.x, bp.y, bp.z);
    if (id < 0 || !blocks[id]) return -1;
    li = (v.x - bp.x * kB) + (v.y - bp.y * kB) * kB + (v.z - bp.z * kB) * kB * kB;
    return id;
  }
  static I3 step(I3 v, int k, int s) { return I3{v.x + (k == 0) * s, v.y + (k == 1) * s, v.z + (k == 2) * s}; }
  // neighbour usable by the masked queries (primal_dual_query.h:90-234):
  // block exists, voxel observed, mask set
  const PDB *pd_usable(I3 v, int &li) const {
    int id = voxel_id(v, li);
    if (id < 0 || blocks[id]->w[li] < (R)1e-6f) return nullptr;
    auto it = pd.find(id);
    if (it == pd.end() || !it->second->mask[li]) return nullptr;
    return it->second.get();
  }
  static R huber(R x, R a) { return std::fabs(x) < a ? (R)0.5f * (x * x) / a : std::fabs(x) - (R)0.5f * a; }

  // PrimalDualInit (optimize/primal_dual.cu:15-40) with GetInitSDFGradient
  // (geometry/primal_dual_query.h:45-87)
  void huber_init() {
    pd.clear();
    for (int id : cand) pd[id].reset(new PDB());
    for (int id : cand) {
      Blk<R> *b = blocks[id].get();
      PDB *s = pd[id].get();
      for (int i = 0; i < kBV; ++i) s->mask[i] = false;
      for (int i = 0; i < kBV; ++i) {
        if (b->w[i] < (R)1e-6f) continue;
        I3 v{b->x * kB + i % kB, b->y * kB + (i / kB) % kB, b->z * kB + i / (kB * kB)};
        V3<R> g = mk((R)0, (R)0, (R)0);
        R q[3];
        bool ok = true;
        for (int k = 0; k < 3 && ok; ++k) {
          int li, nid = voxel_id(step(v, k, 1), li);
          ok = nid >= 0 && blocks[nid]->w[li] >= (R)1e-6f;
          if (ok) q[k] = blocks[nid]->sdf[li];
        }
        if (ok) g = mk(q[0] - b->sdf[i], q[1] - b->sdf[i], q[2] - b->sdf[i]);
        s->w[i] = std::exp(length(g) / vs());
        s->sdf0[i] = b->sdf[i];
        s->bar[i] = 0;
        s->p[i][0] = s->p[i][1] = s->p[i][2] = 0;
        s->mask[i] = true;
      }
    }
  }

  // forward differences of the sdf (bar = false) or of sdf_bar (bar = true)
  // over masked neighbours (GetSDFGradient / GetPrimalGradient,
  // primal_dual_query.h:90-133 and 188-231)
  V3<R> pd_grad(I3 v, R c, bool bar) const {
    R q[3];
    for (int k = 0; k < 3; ++k) {
      int li;
      const PDB *n = pd_usable(step(v, k, 1), li);
      if (!n) return mk((R)0, (R)0, (R)0);
      q[k] = bar ? n->bar[li] : blocks[voxel_id(step(v, k, 1), li)]->sdf[li];
    }
    return mk(q[0] - c, q[1] - c, q[2] - c);
  }

  // PrimalDualIterate (optimize/primal_dual.cu:176-223): pass 1 (dual step and
  // energies, :44-104), then pass 2 (primal step, :106-143), iters times
  void huber_iterate(R lambda, R sigma, R tau, int iters) {
    const R alpha = (R)0.02f;
    for (int it = 0; it < iters; ++it) {
      double ed = 0, et = 0;
      for (int id : cand) {
        auto f = pd.find(id);
        if (f == pd.end()) continue;
        Blk<R> *b = blocks[id].get();
        PDB *s = f->second.get();
        for (int i = 0; i < kBV; ++i) {
          if (b->w[i] < (R)1e-6f || !s->mask[i]) continue;
          I3 v{b->x * kB + i % kB, b->y * kB + (i / kB) % kB, b->z * kB + i / (kB * kB)};
          R dd = std::fabs(b->sdf[i] - s->sdf0[i]);
          ed += (double)(dd * dd);
          et += (double)huber(length(pd_grad(v, b->sdf[i], false)), alpha);
          V3<R> g = pd_grad(v, s->bar[i], true);
          R px = s->p[i][0] + sigma * g.x, py = s->p[i][1] + sigma * g.y, pz = s->p[i][2] + sigma * g.z;
          R h = (R)1 + sigma * alpha;
          px /= h, py /= h, pz /= h;
          R nrm = std::max((R)1, std::sqrt(px * px + py * py + pz * pz));
          s->p[i][0] = px / nrm, s->p[i][1] = py / nrm, s->p[i][2] = pz / nrm;
        }
      }
      pd_err[0] = ed, pd_err[1] = et;
      for (int id : cand) {
        auto f = pd.find(id);
        if (f == pd.end()) continue;
        Blk<R> *b = blocks[id].get();
        PDB *s = f->second.get();
        for (int i = 0; i < kBV; ++i) {
          if (b->w[i] < (R)1e-6f || !s->mask[i]) continue;
          I3 v{b->x * kB + i % kB, b->y * kB + (i / kB) % kB, b->z * kB + i / (kB * kB)};
          // GetDualDivergence (primal_dual_query.h:136-185): backward neighbours
          R div = 0, pn[3];
          bool ok = true;
          for (int k = 0; k < 3 && ok; ++k) {
            int li;
            const PDB *n = pd_usable(step(v, k, -1), li);
            ok = n != nullptr;
            if (ok) pn[k] = n->p[li][k];
          }
          if (ok) div = (pn[0] - s->p[i][0]) + (pn[1] - s->p[i][1]) + (pn[2] - s->p[i][2]);
          R prev = b->sdf[i];
          R lam = lambda * s->w[i];
          R x = prev - tau * div;
          x = (x + lam * tau * s->sdf0[i]) / ((R)1 + lam * tau);
          if (s->w[i] > (R)2) x = s->sdf0[i];
          b->sdf[i] = x;
          s->bar[i] = (R)2 * x - prev;
        }
      }
    }
  }

  // ---------------------------------------------------------- queries
  // GetVoxelValue by voxel coordinate (geometry/voxel_query.h:78-99)
  const Blk<R> *block_of(I3 v, int &li) const {
    I3 bp = voxel_to_block(v);
    int id = find(bp.x, bp.y, bp.z);
    if (id < 0 || !blocks[id]) return nullptr;
    li = (v.x - bp.x * kB) + (v.y - bp.y * kB) * kB + (v.z - bp.z * kB) * kB * kB;
    return blocks[id].get();
  }
  // GetSpatialValue (geometry/spatial_query.h:23-66): trilinear sdf and the
  // interpolated radius; false when any corner block is missing.
  bool spatial(V3<R> pos, R &sdf, R *radius = nullptr) const {
    R off = vs();
    V3<R> pc = mk(pos.x - (R)0.5 * off, pos.y - (R)0.5 * off, pos.z - (R)0.5 * off);
    V3<R> q = world_to_voxelf(pos);
    V3<R> ratio = mk(q.x - std::floor(q.x), q.y - std::floor(q.y), q.z - std::floor(q.z));
    R s = 0, rad = 0;
    for (int i = 0; i < 8; ++i) {
      int mx = (i & 4) > 0, my = (i & 2) > 0, mz = (i & 1) > 0;
      R rx = mx ? ratio.x : (R)1 - ratio.x;
      R ry = my ? ratio.y : (R)1 - ratio.y;
      R rz = mz ? ratio.z : (R)1 - ratio.z;
      V3<R> cw = mk(pc.x + (R)mx * off, pc.y + (R)my * off, pc.z + (R)mz * off);
      I3 v = world_to_voxeli(cw);
      int li;
      const Blk<R> *b = block_of(v, li);
      if (!b) return false;
      R w = rx * ry * rz;
      s += w * b->sdf[li];
      rad += w * std::sqrt((R)1 / b->w[li]);
    }
    sdf = s;
    if (radius) *radius = rad;
    return true;
  }
  // GetSpatialSDFGradient (geometry/spatial_query.h:68-97)
  bool gradient(V3<R> pos, V3<R> &g) const {
    R h = (R)0.5 * vs();
    R sp[3], sn[3];
    for (int i = 0; i < 3; ++i) {
      V3<R> dp = mk(i == 0 ? h : (R)0, i == 1 ? h : (R)0, i == 2 ? h : (R)0);
      if (!spatial(pos - dp, sn[i])) return false;
      if (!spatial(pos + dp, sp[i])) return false;
    }
    g = mk((sp[0] - sn[0]) / vs(), (sp[1] - sn[1]) / vs(), (sp[2] - sn[2]) / vs());
    return true;
  }

  // ---------------------------------------------------------- tracking
  // PointToSurfaceKernel (localizing/point_to_psdf.cu:19-84): over the odd
  // pixels (x and y odd) with a valid depth, the frame point moved to the
  // world by T, its trilinear sdf D and gradient g (both must exist), and
  // J = [g, p x g]; sums of J J^T, D J, D^2 and the count, in double.  The
  // reference writes J[2] = g.x (point_to_psdf.cu:70); fix_j uses g.z.
  void point_to_psdf(const M4<R> &T, bool fix_j, double *A, double *b, double &err, int &count) const {
    for (int i = 0; i < 36; ++i) A[i] = 0.0;
    for (int i = 0; i < 6; ++i) b[i] = 0.0;
    err = 0.0;
    count = 0;
    for (unsigned y = 1; y < p.height; y += 2) {
      for (unsigned x = 1; x < p.width; x += 2) {
        float df = depth[(size_t)y * p.width + x];
        if (depth_invalid(df)) continue;
        V3<R> pc = reproject(x, y, (R)df, (R)p.fx, (R)p.fy, (R)p.cx, (R)p.cy);
        V3<R> pw = T.pt(pc);
        R d;
        V3<R> g;
        if (!spatial(pw, d) || !gradient(pw, g)) continue;
        R J[6] = {g.x, g.y, fix_j ? g.z : g.x, -g.y * pw.z + g.z * pw.y, -g.z * pw.x + g.x * pw.z,
                  -g.x * pw.y + g.y * pw.x};
        for (int i = 0; i < 6; ++i) {
          for (int j = 0; j < 6; ++j) A[i * 6 + j] += (double)(J[i] * J[j]);
          b[i] += (double)(d * J[i]);
        }
        err += (double)(d * d);
        ++count;
      }
    }
  }

  // ---------------------------------------------------------- marching cubes
  // SurfelExtractionKernel (meshing/marching_cubes.cu:75-170): cube validity,
  // cube index, and the shared vertices of cut edges.
  bool corner(I3 v, R &d) const {
    int li;
    const Blk<R> *b = block_of(v, li);
    if (!b) return false;
    d = b->sdf[li];
    if (std::fabs(d) > (R)0.20f) return false;
    R rho = b->a[li] / (b->a[li] + b->b[li]);
    R lim = (R)1 / vs();
    if (rho < (R)0.1f || b->w[li] < lim * lim) return false;
    return true;
  }
  // VertexIntersection (marching_cubes.cu:16-28) with the owner cube's
  // endpoint order: x edge (v+x, v), y edge (v, v+y), z edge (v, v+z).
  void compute_vertex(int ox, int oy, int oz, int slot, Vtx<R> &vt) const {
    I3 v0{ox, oy, oz};
    I3 v1{ox + (slot == 0), oy + (slot == 1), oz + (slot == 2)};
    int li0 = 0, li1 = 0;
    const Blk<R> *b0 = block_of(v0, li0), *b1 = block_of(v1, li1);
    R d0 = b0->sdf[li0], d1 = b1->sdf[li1];
    V3<R> P = voxel_to_world(v0);
    V3<R> q0 = P;
    V3<R> q1 = mk(P.x + vs() * (R)(slot == 0), P.y + vs() * (R)(slot == 1), P.z + vs() * (R)(slot == 2));
    V3<R> p1, p2;
    R e1, e2;
    if (slot == 0) {
      p1 = q1, p2 = q0, e1 = d1, e2 = d0;
    } else {
      p1 = q0, p2 = q1, e1 = d0, e2 = d1;
    }
    V3<R> pos;
    if ((double)std::fabs(e1) < 0.008) {
      pos = p1;
    } else if ((double)std::fabs(e2) < 0.008) {
      pos = p2;
    } else {
      R mu = ((R)0 - e1) / (e2 - e1);
      pos = mk(p1.x + mu * (p2.x - p1.x), p1.y + mu * (p2.y - p1.y), p1.z + mu * (p2.z - p1.z));
    }
    vt.pos[0] = pos.x, vt.pos[1] = pos.y, vt.pos[2] = pos.z;
    R s, rad;
    if (spatial(pos, s, &rad)) {
      R is2 = (R)1 / (rad * rad);
      vt.radius = std::sqrt((R)1 / is2);
    } else {
      vt.radius = 0;
    }
    V3<R> g;
    bool ok = gradient(pos, g);
    R l = length(g);
    if (ok && l > (R)0) {
      vt.normal[0] = g.x / l, vt.normal[1] = g.y / l, vt.normal[2] = g.z / l;
    } else {
      vt.normal[0] = vt.normal[1] = vt.normal[2] = 0;
    }
  }

  void mesh() {
    init_tables();
    ++epoch;
    // pass 1a: cube indices of every candidate cube, list of needed vertices
    int nt = 1;
#ifdef _OPENMP
    nt = omp_get_max_threads();
#endif
    std::vector<std::vector<uint64_t>> need(nt);
#pragma omp parallel for schedule(dynamic, 8)
    for (int ci = 0; ci < (int)cand.size(); ++ci) {
      int tid = 0;
#ifdef _OPENMP
      tid = omp_get_thread_num();
#endif
      Blk<R> *b = blocks[cand[ci]].get();
      for (int i = 0; i < kBV; ++i) {
        int vx = b->x * kB + (i % kB), vy = b->y * kB + (i % (kB * kB)) / kB, vz = b->z * kB + i / (kB * kB);
        int c = 0;
        bool ok = true;
        for (int k = 0; k < 8 && ok; ++k) {
          R d;
          if (!corner(I3{vx + kVtx[k][0], vy + kVtx[k][1], vz + kVtx[k][2]}, d)) ok = false;
          else if (d < (R)0) c |= 1 << k;
        }
        b->cube[i] = ok ? (uint8_t)c : 0;
        if (!ok || c == 0 || c == 255) continue;
        int em = kCaseEdges[c];
        for (int e = 0; e < 12; ++e)
          if (em & (1 << e))
            need[tid].push_back(vkey(vx + kOwner[e][0], vy + kOwner[e][1], vz + kOwner[e][2], kOwner[e][3]));
      }
    }
    std::vector<uint64_t> nk;
    for (auto &v : need) nk.insert(nk.end(), v.begin(), v.end());
    std::sort(nk.begin(), nk.end());
    nk.erase(std::unique(nk.begin(), nk.end()), nk.end());
    // pass 1b: create and (re)compute each needed vertex once
    std::vector<Vtx<R> *> vp(nk.size());
    for (size_t j = 0; j < nk.size(); ++j) vp[j] = &verts[nk[j]];
#pragma omp parallel for schedule(dynamic, 64)
    for (long j = 0; j < (long)nk.size(); ++j) {
      uint64_t k = nk[j];
      compute_vertex(sext20(k >> 42), sext20(k >> 22), sext20(k >> 2), (int)(k & 3), *vp[j]);
      vp[j]->epoch = epoch;
    }
    // pass 2: surfel counts and triangle (re)assignment
    // TriangleExtractionKernel (marching_cubes.cu:180-275)
    for (int ci = 0; ci < (int)cand.size(); ++ci) {
      Blk<R> *b = blocks[cand[ci]].get();
      b->inner = b->boundary = 0;
      for (int i = 0; i < kBV; ++i) {
        int ox = i % kB, oy = (i % (kB * kB)) / kB, oz = i / (kB * kB);
        int vx = b->x * kB + ox, vy = b->y * kB + oy, vz = b->z * kB + oz;
        bool in = ox >= 1 && oy >= 1 && oz >= 1 && ox < kB - 1 && oy < kB - 1 && oz < kB - 1;
        for (int s = 0; s < 3; ++s)
          if (verts.count(vkey(vx, vy, vz, s))) (in ? b->inner : b->boundary)++;
      }
    }
    for (int ci = 0; ci < (int)cand.size(); ++ci) {
      Blk<R> *b = blocks[cand[ci]].get();
      for (int i = 0; i < kBV; ++i) {
        int c = b->cube[i];
        if (c == 0 || c == 255) continue;
        int vx = b->x * kB + (i % kB), vy = b->y * kB + (i % (kB * kB)) / kB, vz = b->z * kB + i / (kB * kB);
        uint64_t ev[12];
        for (int e = 0; e < 12; ++e)
          ev[e] = vkey(vx + kOwner[e][0], vy + kOwner[e][1], vz + kOwner[e][2], kOwner[e][3]);
        Tris &T = tris[vkey(vx, vy, vz, 0)];
        int n = case_tri_count(c);
        for (int t = 0; t < n; ++t) {
          if (t < T.n) {
            for (int q = 0; q < 3; ++q) verts[T.v[t][q]].ref -= 1;
          }
          for (int q = 0; q < 3; ++q) {
            T.v[t][q] = ev[case_edge(c, 3 * t + q)];
            verts[T.v[t][q]].ref += 1;
          }
        }
        if (n > T.n) T.n = (uint8_t)n;
      }
    }
    // RecycleTrianglesKernel (marching_cubes.cu:278-301)
    for (int ci = 0; ci < (int)cand.size(); ++ci) {
      Blk<R> *b = blocks[cand[ci]].get();
      for (int i = 0; i < kBV; ++i) {
        int vx = b->x * kB + (i % kB), vy = b->y * kB + (i % (kB * kB)) / kB, vz = b->z * kB + i / (kB * kB);
        auto it = tris.find(vkey(vx, vy, vz, 0));
        if (it == tris.end()) continue;
        int n = case_tri_count(b->cube[i]);
        Tris &T = it->second;
        for (int t = n; t < T.n; ++t)
          for (int q = 0; q < 3; ++q) verts[T.v[t][q]].ref -= 1;
        if (n < T.n) T.n = (uint8_t)n;
        if (T.n == 0) tris.erase(it);
      }
    }
    // RecycleVerticesKernel (marching_cubes.cu:303-321)
    for (int ci = 0; ci < (int)cand.size(); ++ci) {
      Blk<R> *b = blocks[cand[ci]].get();
      for (int i = 0; i < kBV; ++i) {
        int vx = b->x * kB + (i % kB), vy = b->y * kB + (i % (kB * kB)) / kB, vz = b->z * kB + i / (kB * kB);
        for (int s = 0; s < 3; ++s) {
          auto it = verts.find(vkey(vx, vy, vz, s));
          if (it != verts.end() && it->second.ref == 0) verts.erase(it);
        }
      }
    }
  }

  // ---------------------------------------------------------- raycast
  // CastKernel (visualization/ray_caster.cu:16-150) and BisectionIntersection
  // (geometry/isosurface_intersection.h:21-55).
  //
  // The march is a chain of discrete decisions (sample validity, sign change,
  // regula-falsi side), so it always runs in single precision, recording the
  // decisions.  In FP64 mode the hit is then re-evaluated in double along the
  // same decisions: the two bracketing samples and the regula-falsi steps use
  // double positions and double trilinear values.
  struct Trace {
    bool hit = false;
    float t0 = 0, t1 = 0;   // bracketing samples
    uint8_t side = 0;       // bit k: iteration k moved the left end
  };

  template <class T>
  bool spatial_t(V3<T> pos, T &sdf) const {
    T off = (T)p.voxel_size;
    V3<T> pc = mk(pos.x - (T)0.5 * off, pos.y - (T)0.5 * off, pos.z - (T)0.5 * off);
    V3<T> q = pos / off;
    V3<T> ratio = mk(q.x - std::floor(q.x), q.y - std::floor(q.y), q.z - std::floor(q.z));
    T s = 0;
    for (int i = 0; i < 8; ++i) {
      int mx = (i & 4) > 0, my = (i & 2) > 0, mz = (i & 1) > 0;
      T rx = mx ? ratio.x : (T)1 - ratio.x;
      T ry = my ? ratio.y : (T)1 - ratio.y;
      T rz = mz ? ratio.z : (T)1 - ratio.z;
      V3<T> cw = mk(pc.x + (T)mx * off, pc.y + (T)my * off, pc.z + (T)mz * off);
      auto rnd = [&](T v) { T sg = v < (T)0 ? (T)-1 : (T)1; return f2i<T>(v / off + sg * (T)0.5); };
      I3 v{rnd(cw.x), rnd(cw.y), rnd(cw.z)};
      int li;
      const Blk<R> *b = block_of(v, li);
      if (!b) return false;
      s += (rx * ry * rz) * (T)b->sdf[li];
    }
    sdf = s;
    return true;
  }

  // FP64 sample along a single-precision path: the cell choice (the corner
  // voxels from rounding p - v/2 and the floor of p/v, two separate discrete
  // results in GetSpatialValue) is taken from the single-precision position
  // p32; the fractional weights and the sum are evaluated in R at p.
  bool spatial_hyb(V3<R> pos, V3<float> p32, R &sdf) const {
    const float off = p.voxel_size;
    V3<float> pc = mk(p32.x - 0.5f * off, p32.y - 0.5f * off, p32.z - 0.5f * off);
    V3<float> q32 = p32 / off;
    const float fl[3] = {std::floor(q32.x), std::floor(q32.y), std::floor(q32.z)};
    const R vs = (R)p.voxel_size;
    const R ratio[3] = {pos.x / vs - (R)fl[0], pos.y / vs - (R)fl[1], pos.z / vs - (R)fl[2]};
    auto rnd = [&](float v) { float sg = v < 0.0f ? -1.0f : 1.0f; return f2i<float>(v / off + sg * 0.5f); };
    R s = 0;
    for (int i = 0; i < 8; ++i) {
      int mx = (i & 4) > 0, my = (i & 2) > 0, mz = (i & 1) > 0;
      R rx = mx ? ratio[0] : (R)1 - ratio[0];
      R ry = my ? ratio[1] : (R)1 - ratio[1];
      R rz = mz ? ratio[2] : (R)1 - ratio[2];
      I3 v{rnd(pc.x + (float)mx * off), rnd(pc.y + (float)my * off), rnd(pc.z + (float)mz * off)};
      int li;
      const Blk<R> *b = block_of(v, li);
      if (!b) return false;
      s += (rx * ry * rz) * (R)b->sdf[li];
    }
    sdf = s;
    return true;
  }

  Trace march32(const M4<float> &wTcf, int x, int y) const {
    Trace tr;
    const float fx = p.rc_fx, fy = p.rc_fy, cx = p.rc_cx, cy = p.rc_cy;
    V3<float> cd = normalize(mk(((float)x - cx) / fx, ((float)y - cy) / fy, 1.0f));
    float tmin = p.min_raycast_depth / cd.z, tmax = p.max_raycast_depth / cd.z;
    V3<float> cam = wTcf.pt(mk(0.0f, 0.0f, 0.0f));
    V3<float> wd = normalize(wTcf.dir(cd));
    bool have_prev = false;
    float prev_sdf = 0, prev_t = 0;
    for (float t = tmin; t < tmax; t += p.raycast_step) {
      float s;
      if (!spatial_t<float>(cam + t * wd, s)) continue;
      if (have_prev && prev_sdf > 0.0f && s < 0.0f) {
        float l = prev_t, r = t, ls = prev_sdf, rs = s;
        bool found = true;
        uint8_t side = 0;
        for (int k = 0; k < 3; ++k) {
          float m = l + (ls / (ls - rs)) * (r - l);
          float ms;
          if (!spatial_t<float>(cam + m * wd, ms)) {
            found = false;
            break;
          }
          if ((double)(ls * ms) > 0.0) {
            l = m, ls = ms, side |= 1 << k;
          } else {
            r = m, rs = ms;
          }
        }
        if (found && std::fabs(prev_sdf - s) < p.sample_sdf_threshold && std::fabs(s) < p.sdf_threshold) {
          tr.hit = true, tr.t0 = prev_t, tr.t1 = t, tr.side = side;
          return tr;
        }
      }
      prev_sdf = s, prev_t = t, have_prev = true;
    }
    return tr;
  }

  // diagnostic: the single-precision trace of one pixel and the values the
  // replay sees (out: t0, t1, side, s32(t0), s32(t1), sR(t0), sR(t1), m per step)
  void debug_ray(const M4<R> &cTw_, int x, int y, double *out) const {
    M4<float> cf;
    for (int i = 0; i < 16; ++i) cf.e[i] = (float)cTw_.e[i];
    const M4<float> wf = inverse(cf);
    Trace tr = march32(wf, x, y);
    for (int k = 0; k < 16; ++k) out[k] = 0;
    out[0] = tr.hit, out[1] = tr.t0, out[2] = tr.t1, out[3] = tr.side;
    if (!tr.hit) return;
    V3<float> cdf = normalize(mk(((float)x - p.rc_cx) / p.rc_fx, ((float)y - p.rc_cy) / p.rc_fy, 1.0f));
    V3<float> camf = wf.pt(mk(0.0f, 0.0f, 0.0f));
    V3<float> wdf = normalize(wf.dir(cdf));
    float a, b;
    spatial_t<float>(camf + tr.t0 * wdf, a);
    spatial_t<float>(camf + tr.t1 * wdf, b);
    out[4] = a, out[5] = b;
    const M4<R> wt = inverse(cTw_);
    V3<R> cd = normalize(mk(((R)x - (R)p.rc_cx) / (R)p.rc_fx, ((R)y - (R)p.rc_cy) / (R)p.rc_fy, (R)1));
    V3<R> cam = wt.pt(mk((R)0, (R)0, (R)0));
    V3<R> wd = normalize(wt.dir(cd));
    R ls, rs;
    spatial_t<R>(cam + (R)tr.t0 * wd, ls);
    spatial_t<R>(cam + (R)tr.t1 * wd, rs);
    out[6] = ls, out[7] = rs;
    float l = tr.t0, r = tr.t1, lsf = a, rsf = b;
    for (int k = 0; k < 3; ++k) {
      float m = l + (lsf / (lsf - rsf)) * (r - l);
      float ms;
      spatial_t<float>(camf + m * wdf, ms);
      out[8 + 2 * k] = m, out[9 + 2 * k] = ms;
      if ((double)(lsf * ms) > 0.0) l = m, lsf = ms;
      else r = m, rsf = ms;
    }
  }

  void raycast(const M4<R> &cTw_, float *odepth, float *overt, float *onorm) const {
    M4<float> cf;
    for (int i = 0; i < 16; ++i) cf.e[i] = (float)cTw_.e[i];
    const M4<float> wf = inverse(cf);
    const M4<R> wTc_ = sizeof(R) == 4 ? M4<R>{} : inverse(cTw_);
    int W = p.rc_width, H = p.rc_height;
#pragma omp parallel for schedule(dynamic, 2)
    for (int y = 0; y < H; ++y) {
      for (int x = 0; x < W; ++x) {
        size_t pix = (size_t)y * W + x;
        const float NI = -INFINITY;
        if (odepth) odepth[pix] = NI;
        if (overt) for (int k = 0; k < 4; ++k) overt[4 * pix + k] = NI;
        if (onorm) for (int k = 0; k < 4; ++k) onorm[4 * pix + k] = NI;
        Trace tr = march32(wf, x, y);
        if (!tr.hit) continue;
        // evaluate the hit along the recorded decisions: the single-precision
        // regula falsi runs in lockstep to supply the discrete cell choices
        M4<R> wt;
        for (int i = 0; i < 16; ++i) wt.e[i] = sizeof(R) == 4 ? (R)wf.e[i] : wTc_.e[i];
        const R fx = p.rc_fx, fy = p.rc_fy, cx = p.rc_cx, cy = p.rc_cy;
        const R rx = ((R)x - cx) / fx, ry = ((R)y - cy) / fy;
        V3<R> cd = normalize(mk(rx, ry, (R)1));
        V3<R> cam = wt.pt(mk((R)0, (R)0, (R)0));
        V3<R> wd = normalize(wt.dir(cd));
        V3<float> cdf = normalize(mk(((float)x - p.rc_cx) / p.rc_fx, ((float)y - p.rc_cy) / p.rc_fy, 1.0f));
        V3<float> camf = wf.pt(mk(0.0f, 0.0f, 0.0f));
        V3<float> wdf = normalize(wf.dir(cdf));
        float l32 = tr.t0, r32 = tr.t1, ls32, rs32;
        spatial_t<float>(camf + l32 * wdf, ls32);
        spatial_t<float>(camf + r32 * wdf, rs32);
        R l = tr.t0, r = tr.t1, ls, rs, m = 0;
        if (!spatial_hyb(cam + l * wd, camf + l32 * wdf, ls) || !spatial_hyb(cam + r * wd, camf + r32 * wdf, rs))
          continue;
        bool ok = true;
        for (int k = 0; k < 3; ++k) {
          const float m32 = l32 + (ls32 / (ls32 - rs32)) * (r32 - l32);
          m = l + (ls / (ls - rs)) * (r - l);
          float ms32;
          R ms;
          spatial_t<float>(camf + m32 * wdf, ms32);
          if (!spatial_hyb(cam + m * wd, camf + m32 * wdf, ms)) {
            ok = false;
            break;
          }
          // a value whose sign contradicts the recorded single-precision
          // decision is within rounding of zero: the root is at m
          const bool left = (tr.side >> k) & 1;
          if (left != ((double)(ls * ms) > 0.0)) ms = 0;
          if (left) {
            l = m, ls = ms, l32 = m32, ls32 = ms32;
          } else {
            r = m, rs = ms, r32 = m32, rs32 = ms32;
          }
        }
        if (!ok) continue;
        R dz = m * cd.z;
        if (odepth) odepth[pix] = (float)dz;
        if (overt) {
          overt[4 * pix] = (float)(dz * rx), overt[4 * pix + 1] = (float)(dz * ry);
          overt[4 * pix + 2] = (float)dz, overt[4 * pix + 3] = 1.0f;
        }
        if (p.enable_gradients && onorm) {
          V3<R> iso = cam + m * wd;
          V3<R> g;
          bool gok = gradient(iso, g);
          R len = length(g);
          V3<R> n = (gok && len > (R)0) ? g / len : mk((R)0, (R)0, (R)0);
          n = mk(-n.x, -n.y, -n.z);
          V3<R> nc = cTw_.dir(n);
          onorm[4 * pix] = (float)nc.x, onorm[4 * pix + 1] = (float)nc.y;
          onorm[4 * pix + 2] = (float)nc.z, onorm[4 * pix + 3] = 1.0f;
        }
      }
    }
  }

  // ---------------------------------------------------------- raycast backward
  // Reverse-mode derivative of the raycast above (the library's
  // mh_raycast_backward restated): along the recorded single-precision
  // decisions, the depth m * cd.z is differentiated through the bracketing
  // samples, the three regula-falsi steps and the gradient-based normal, for
  // the voxel sdf values and a left se(3) increment of wTc (translation
  // first).  Samples keep the hybrid cell choice of spatial_hyb.
  struct SampD {
    R s = 0;
    V3<R> g{0, 0, 0};
    int id[8];
    int li[8];
    R w[8];
  };
  bool spatial_d(V3<R> pos, V3<float> p32, SampD &o) const {
    const float off = p.voxel_size;
    V3<float> pc = mk(p32.x - 0.5f * off, p32.y - 0.5f * off, p32.z - 0.5f * off);
    V3<float> q32 = p32 / off;
    const float fl[3] = {std::floor(q32.x), std::floor(q32.y), std::floor(q32.z)};
    const R vsr = (R)p.voxel_size;
    const R ratio[3] = {pos.x / vsr - (R)fl[0], pos.y / vsr - (R)fl[1], pos.z / vsr - (R)fl[2]};
    auto rnd = [&](float v) { float sg = v < 0.0f ? -1.0f : 1.0f; return f2i<float>(v / off + sg * 0.5f); };
    R sum = 0, gx = 0, gy = 0, gz = 0;
    for (int i = 0; i < 8; ++i) {
      int mx = (i & 4) > 0, my = (i & 2) > 0, mz = (i & 1) > 0;
      R rx = mx ? ratio[0] : (R)1 - ratio[0];
      R ry = my ? ratio[1] : (R)1 - ratio[1];
      R rz = mz ? ratio[2] : (R)1 - ratio[2];
      I3 v{rnd(pc.x + (float)mx * off), rnd(pc.y + (float)my * off), rnd(pc.z + (float)mz * off)};
      I3 bp = voxel_to_block(v);
      int bid = find(bp.x, bp.y, bp.z);
      if (bid < 0 || !blocks[bid]) return false;
      int li = (v.x - bp.x * kB) + (v.y - bp.y * kB) * kB + (v.z - bp.z * kB) * kB * kB;
      R val = (R)blocks[bid]->sdf[li];
      sum += (rx * ry * rz) * val;
      gx += (mx ? (R)1 : (R)-1) * ry * rz * val;
      gy += (my ? (R)1 : (R)-1) * rx * rz * val;
      gz += (mz ? (R)1 : (R)-1) * rx * ry * val;
      o.id[i] = bid, o.li[i] = li, o.w[i] = rx * ry * rz;
    }
    o.s = sum;
    o.g = mk(gx / vsr, gy / vsr, gz / vsr);
    return true;
  }
  std::unordered_map<int, std::vector<double>> grad;
  void scatter(const SampD &o, R a) {
    if (a == (R)0) return;
    for (int i = 0; i < 8; ++i) {
      auto &g = grad[o.id[i]];
      if (g.empty()) g.assign(kBV, 0.0);
      g[o.li[i]] += (double)(a * o.w[i]);
    }
  }
  static V3<R> cross(V3<R> a, V3<R> b) {
    return mk(a.y * b.z - a.z * b.y, a.z * b.x - a.x * b.z, a.x * b.y - a.y * b.x);
  }
  // dL_dD: W x H, dL_dN: W x H x 3 (may be null); xi receives dL/dxi
  void raycast_backward(const M4<R> &cTw_, const float *dL_dD, const float *dL_dN, double xi[6]) {
    grad.clear();
    for (int k = 0; k < 6; ++k) xi[k] = 0;
    M4<float> cf;
    for (int i = 0; i < 16; ++i) cf.e[i] = (float)cTw_.e[i];
    const M4<float> wf = inverse(cf);
    const M4<R> wTc_ = sizeof(R) == 4 ? M4<R>{} : inverse(cTw_);
    M4<R> wt;
    for (int i = 0; i < 16; ++i) wt.e[i] = sizeof(R) == 4 ? (R)wf.e[i] : wTc_.e[i];
    const int W = p.rc_width, H = p.rc_height;
    const R vsr = (R)p.voxel_size;
    for (int y = 0; y < H; ++y) {
      for (int x = 0; x < W; ++x) {
        const size_t pix = (size_t)y * W + x;
        R aD = dL_dD ? (R)dL_dD[pix] : (R)0;
        V3<R> aN = dL_dN ? mk((R)dL_dN[3 * pix], (R)dL_dN[3 * pix + 1], (R)dL_dN[3 * pix + 2]) : mk((R)0, (R)0, (R)0);
        if (aD == (R)0 && aN.x == (R)0 && aN.y == (R)0 && aN.z == (R)0) continue;
        Trace tr = march32(wf, x, y);
        if (!tr.hit) continue;
        const R rx = ((R)x - (R)p.rc_cx) / (R)p.rc_fx, ry = ((R)y - (R)p.rc_cy) / (R)p.rc_fy;
        V3<R> cd = normalize(mk(rx, ry, (R)1));
        V3<R> cam = wt.pt(mk((R)0, (R)0, (R)0));
        V3<R> wd = normalize(wt.dir(cd));
        V3<float> cdf = normalize(mk(((float)x - p.rc_cx) / p.rc_fx, ((float)y - p.rc_cy) / p.rc_fy, 1.0f));
        V3<float> camf = wf.pt(mk(0.0f, 0.0f, 0.0f));
        V3<float> wdf = normalize(wf.dir(cdf));
        // forward along the recorded decisions
        SampD S0, S1, Sm[3];
        float l32 = tr.t0, r32 = tr.t1, ls32, rs32;
        spatial_t<float>(camf + l32 * wdf, ls32);
        spatial_t<float>(camf + r32 * wdf, rs32);
        R l = tr.t0, r = tr.t1;
        if (!spatial_d(cam + l * wd, camf + l32 * wdf, S0) || !spatial_d(cam + r * wd, camf + r32 * wdf, S1)) continue;
        R ls = S0.s, rs = S1.s;
        R L[3], Rr[3], LS[3], RS[3], M[3];
        bool zero[3] = {false, false, false}, ok = true;
        for (int k = 0; k < 3; ++k) {
          L[k] = l, Rr[k] = r, LS[k] = ls, RS[k] = rs;
          const float m32 = l32 + (ls32 / (ls32 - rs32)) * (r32 - l32);
          const R m = l + (ls / (ls - rs)) * (r - l);
          M[k] = m;
          float ms32;
          spatial_t<float>(camf + m32 * wdf, ms32);
          if (!spatial_d(cam + m * wd, camf + m32 * wdf, Sm[k])) {
            ok = false;
            break;
          }
          R ms = Sm[k].s;
          const bool left = (tr.side >> k) & 1;
          if (left != ((double)(ls * ms) > 0.0)) ms = 0, zero[k] = true;
          if (left) l = m, ls = ms, l32 = m32, ls32 = ms32;
          else r = m, rs = ms, r32 = m32, rs32 = ms32;
        }
        if (!ok) continue;
        const R m = M[2];
        V3<R> a_cam = mk((R)0, (R)0, (R)0), a_wd = a_cam, a_w = a_cam;
        R am = aD * cd.z;
        if (dL_dN && (aN.x != (R)0 || aN.y != (R)0 || aN.z != (R)0)) {
          V3<R> iso = cam + m * wd;
          const R h = (R)0.5 * vsr;
          SampD P[3], N[3];
          bool gok = true;
          for (int i = 0; i < 3 && gok; ++i) {
            V3<R> dp = mk(i == 0 ? h : (R)0, i == 1 ? h : (R)0, i == 2 ? h : (R)0);
            V3<R> a = iso - dp, b = iso + dp;
            gok = spatial_d(a, mk((float)a.x, (float)a.y, (float)a.z), N[i]) &&
                  spatial_d(b, mk((float)b.x, (float)b.y, (float)b.z), P[i]);
          }
          V3<R> g = mk((P[0].s - N[0].s) / vsr, (P[1].s - N[1].s) / vsr, (P[2].s - N[2].s) / vsr);
          R len = std::sqrt(dot(g, g));
          if (gok && len > (R)0) {
            V3<R> u = g / len, nn = mk(-u.x, -u.y, -u.z);
            const R *c = cTw_.e;
            V3<R> a_nn = mk(c[0] * aN.x + c[4] * aN.y + c[8] * aN.z, c[1] * aN.x + c[5] * aN.y + c[9] * aN.z,
                            c[2] * aN.x + c[6] * aN.y + c[10] * aN.z);
            a_w = cross(a_nn, nn);
            V3<R> a_u = mk(-a_nn.x, -a_nn.y, -a_nn.z);
            R ua = dot(u, a_u);
            R ag[3] = {(a_u.x - u.x * ua) / len, (a_u.y - u.y * ua) / len, (a_u.z - u.z * ua) / len};
            V3<R> a_iso = mk((R)0, (R)0, (R)0);
            for (int i = 0; i < 3; ++i) {
              R ap = ag[i] / vsr, an = -ag[i] / vsr;
              scatter(P[i], ap);
              scatter(N[i], an);
              a_iso = a_iso + ap * P[i].g + an * N[i].g;
            }
            a_cam = a_cam + a_iso;
            a_wd = a_wd + m * a_iso;
            am += dot(a_iso, wd);
          }
        }
        R al = 0, ar = 0, als = 0, ars = 0;
        for (int k = 2; k >= 0; --k) {
          const bool left = (tr.side >> k) & 1;
          R a_mk = (k == 2 ? am : (R)0) + (left ? al : ar);
          R a_ms = left ? als : ars;
          if (left) al = 0, als = 0;
          else ar = 0, ars = 0;
          if (zero[k]) a_ms = 0;   // the value was taken as exactly zero
          scatter(Sm[k], a_ms);
          V3<R> ap = a_ms * Sm[k].g;
          a_cam = a_cam + ap;
          a_wd = a_wd + M[k] * ap;
          a_mk += dot(ap, wd);
          const R den = LS[k] - RS[k], q = LS[k] / den, span = Rr[k] - L[k];
          al += a_mk * ((R)1 - q);
          ar += a_mk * q;
          als += a_mk * span * (-RS[k]) / (den * den);
          ars += a_mk * span * LS[k] / (den * den);
        }
        scatter(S0, als);
        scatter(S1, ars);
        V3<R> p0 = als * S0.g, p1 = ars * S1.g;
        a_cam = a_cam + p0 + p1;
        a_wd = a_wd + (R)tr.t0 * p0 + (R)tr.t1 * p1;
        V3<R> aw = cross(cam, a_cam) + cross(wd, a_wd) + a_w;
        xi[0] += a_cam.x, xi[1] += a_cam.y, xi[2] += a_cam.z;
        xi[3] += aw.x, xi[4] += aw.y, xi[5] += aw.z;
      }
    }
  }
  // per pixel: hit, side, and the bits of t0, t1 of the single-precision trace
  void trace_dump(const M4<R> &cTw_, int32_t *out) const {
    M4<float> cf;
    for (int i = 0; i < 16; ++i) cf.e[i] = (float)cTw_.e[i];
    const M4<float> wf = inverse(cf);
    const int W = p.rc_width, H = p.rc_height;
#pragma omp parallel for schedule(dynamic, 2)
    for (int y = 0; y < H; ++y)
      for (int x = 0; x < W; ++x) {
        Trace tr = march32(wf, x, y);
        int32_t *o = out + 4 * ((size_t)y * W + x);
        o[0] = tr.hit, o[1] = tr.side;
        memcpy(o + 2, &tr.t0, 4);
        memcpy(o + 3, &tr.t1, 4);
      }
  }

  // ---------------------------------------------------------- GC
  // CollectLowSurfelBlocksKernel (mapping/recycle.cu:79-114)
  void gc_low_surfel() {
    for (int id : cand) {
      Blk<R> *b = blocks[id].get();
      b->flag = 0;
      if (b->inner < 10 && b->boundary == 0) b->life--;
      else b->life = kBlockLife;
    }
    static const int nb[6][3] = {{0, 0, 1}, {0, 0, -1}, {0, 1, 0}, {0, -1, 0}, {1, 0, 0}, {-1, 0, 0}};
    for (int id : cand) {
      Blk<R> *b = blocks[id].get();
      if (b->life > 0) continue;
      bool ok = true;
      for (int j = 0; j < 6 && ok; ++j) {
        int q = find(b->x + nb[j][0], b->y + nb[j][1], b->z + nb[j][2]);
        if (q < 0 || !blocks[q]) continue;
        if (blocks[q]->life != 0) ok = false;
      }
      if (ok) b->flag = 1;
    }
  }
  // StarveOccupiedBlocksKernel (recycle.cu:15-25)
  void gc_starve() {
    for (int id : cand) {
      Blk<R> *b = blocks[id].get();
      for (int i = 0; i < kBV; ++i) b->w[i] = std::max((R)0, b->w[i] - (R)1);
    }
  }
  // CollectGarbageBlockArrayKernel (recycle.cu:28-75)
  void gc_collect_garbage() {
    for (int id : cand) {
      Blk<R> *b = blocks[id].get();
      R mn = INFINITY, mx = 0;
      for (int i = 0; i < kBV; ++i) {
        R s = (double)b->w[i] < 1e-6 ? (R)INFINITY : b->sdf[i];
        mn = std::min(mn, std::fabs(s));
        mx = std::max(mx, b->w[i]);
      }
      R t = truncate((R)5);
      b->flag = (mn >= t || (double)mx < 1e-6) ? 1 : 0;
    }
  }
  // RecycleGarbageTrianglesKernel / RecycleGarbageVerticesKernel
  // (recycle.cu:117-181) followed by HashTable::FreeEntry
  int gc_recycle() {
    for (int id : cand) {
      Blk<R> *b = blocks[id].get();
      if (!b->flag) continue;
      for (int i = 0; i < kBV; ++i) {
        int vx = b->x * kB + (i % kB), vy = b->y * kB + (i % (kB * kB)) / kB, vz = b->z * kB + i / (kB * kB);
        auto it = tris.find(vkey(vx, vy, vz, 0));
        if (it == tris.end()) continue;
        Tris &T = it->second;
        for (int t = 0; t < T.n; ++t)
          for (int q = 0; q < 3; ++q) verts[T.v[t][q]].ref -= 1;
        tris.erase(it);
      }
    }
    int freed = 0;
    std::vector<int> dead;
    for (int id : cand) {
      Blk<R> *b = blocks[id].get();
      if (!b->flag) continue;
      int live = 0;
      for (int i = 0; i < kBV; ++i) {
        int vx = b->x * kB + (i % kB), vy = b->y * kB + (i % (kB * kB)) / kB, vz = b->z * kB + i / (kB * kB);
        for (int s = 0; s < 3; ++s) {
          auto it = verts.find(vkey(vx, vy, vz, s));
          if (it == verts.end()) continue;
          if (it->second.ref <= 0) verts.erase(it);
          else ++live;
        }
      }
      if (live == 0) dead.push_back(id);
    }
    for (int id : dead) {
      erase(id);
      ++freed;
    }
    if (freed) {
      std::vector<int> c2;
      for (int id : cand)
        if (blocks[id]) c2.push_back(id);
      cand.swap(c2);
    }
    return freed;
  }
};

}  // namespace orc

// =================================================================== C API
using namespace orc;

struct OHandle {
  int fp64;
  void *v;
};

template <class R> static Vol<R> *V(OHandle *h) { return (Vol<R> *)h->v; }

#define DISPATCH(h, ...)                  \
  do {                                    \
    if ((h)->fp64) {                      \
      auto *vol = V<double>(h);           \
      __VA_ARGS__;                        \
    } else {                              \
      auto *vol = V<float>(h);            \
      __VA_ARGS__;                        \
    }                                     \
  } while (0)

extern "C" {

void *orc_create(const mh_params *p, int fp64) {
  init_tables();
  OHandle *h = new OHandle;
  h->fp64 = fp64;
  if (fp64) {
    auto *v = new Vol<double>;
    v->p = *p;
    h->v = v;
  } else {
    auto *v = new Vol<float>;
    v->p = *p;
    h->v = v;
  }
  return h;
}

void orc_destroy(void *hp) {
  OHandle *h = (OHandle *)hp;
  if (h->fp64) delete V<double>(h);
  else delete V<float>(h);
  delete h;
}

int orc_num_threads(void) {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}
void orc_set_threads(int n) {
#ifdef _OPENMP
  if (n > 0) omp_set_num_threads(n);
#else
  (void)n;
#endif
}

uint32_t orc_hash_bucket(int x, int y, int z, uint32_t bc) { return hash_bucket(x, y, z, bc); }

void orc_inverse(const float *m, float *out) {
  M4<float> a;
  for (int i = 0; i < 16; ++i) a.e[i] = m[i];
  M4<float> r = inverse(a);
  for (int i = 0; i < 16; ++i) out[i] = r.e[i];
}

void orc_frame_set(void *hp, const float *depth, const float *wTc) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->frame_set(depth, wTc));
}

// Allocation: returns the number of touched blocks.
int orc_allocate(void *hp) {
  OHandle *h = (OHandle *)hp;
  int n = 0;
  DISPATCH(h, n = (int)vol->allocate().size());
  return n;
}
// Blocks touched by the last allocation (sorted by key); writes up to max.
int orc_get_touched(void *hp, int32_t *out_pos, int max) {
  OHandle *h = (OHandle *)hp;
  std::vector<uint64_t> keys;
  DISPATCH(h, keys = vol->touched);
  int n = (int)keys.size();
  for (int i = 0; i < n && i < max && out_pos; ++i) {
    I3 b = unkey(keys[i]);
    out_pos[3 * i] = b.x, out_pos[3 * i + 1] = b.y, out_pos[3 * i + 2] = b.z;
  }
  return n;
}

int orc_collect_frustum(void *hp) {
  OHandle *h = (OHandle *)hp;
  int n = 0;
  DISPATCH(h, { vol->collect_frustum(); n = (int)vol->cand.size(); });
  return n;
}
int orc_collect_all(void *hp) {
  OHandle *h = (OHandle *)hp;
  int n = 0;
  DISPATCH(h, { vol->collect_all(); n = (int)vol->cand.size(); });
  return n;
}

int orc_get_candidates(void *hp, int32_t *pos, int max) {
  OHandle *h = (OHandle *)hp;
  int n = 0;
  DISPATCH(h, {
    n = (int)vol->cand.size();
    for (int i = 0; i < n && i < max; ++i) {
      auto *b = vol->blocks[vol->cand[i]].get();
      pos[3 * i] = b->x, pos[3 * i + 1] = b->y, pos[3 * i + 2] = b->z;
    }
  });
  return n;
}

int orc_set_candidates(void *hp, int n, const int32_t *pos) {
  OHandle *h = (OHandle *)hp;
  int bad = 0;
  DISPATCH(h, {
    vol->cand.clear();
    for (int i = 0; i < n; ++i) {
      int id = vol->find(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      if (id < 0) ++bad;
      else vol->cand.push_back(id);
    }
  });
  return bad;
}

int orc_block_count(void *hp) {
  OHandle *h = (OHandle *)hp;
  int n = 0;
  DISPATCH(h, { n = (int)vol->index.size(); });
  return n;
}

// Dump in key order: pos[3n], fields [512n]; any field pointer may be NULL.
int orc_get_blocks(void *hp, int max, int32_t *pos, float *sdf, float *w, float *a, float *b) {
  OHandle *h = (OHandle *)hp;
  int n = 0;
  DISPATCH(h, {
    std::vector<std::pair<uint64_t, int>> ks(vol->index.begin(), vol->index.end());
    std::sort(ks.begin(), ks.end());
    n = (int)ks.size();
    for (int i = 0; i < n && i < max; ++i) {
      auto *bl = vol->blocks[ks[i].second].get();
      if (pos) pos[3 * i] = bl->x, pos[3 * i + 1] = bl->y, pos[3 * i + 2] = bl->z;
      for (int k = 0; k < kBV; ++k) {
        if (sdf) sdf[(size_t)i * kBV + k] = (float)bl->sdf[k];
        if (w) w[(size_t)i * kBV + k] = (float)bl->w[k];
        if (a) a[(size_t)i * kBV + k] = (float)bl->a[k];
        if (b) b[(size_t)i * kBV + k] = (float)bl->b[k];
      }
    }
  });
  return n;
}

// Load voxel state (inserting blocks as needed).
void orc_set_blocks(void *hp, int n, const int32_t *pos, const float *sdf, const float *w, const float *a,
                    const float *b) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    for (int i = 0; i < n; ++i) {
      int id = vol->insert(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      auto *bl = vol->blocks[id].get();
      for (int k = 0; k < kBV; ++k) {
        if (sdf) bl->sdf[k] = sdf[(size_t)i * kBV + k];
        if (w) bl->w[k] = w[(size_t)i * kBV + k];
        if (a) bl->a[k] = a[(size_t)i * kBV + k];
        if (b) bl->b[k] = b[(size_t)i * kBV + k];
      }
    }
  });
}

void orc_integrate_simple(void *hp) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->integrate_simple());
}
void orc_predict_inlier(void *hp) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->predict_inlier());
}
void orc_integrate_psdf(void *hp) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->integrate_psdf());
}
void orc_get_inlier(void *hp, float *out) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, memcpy(out, vol->inlier.data(), vol->inlier.size() * 4));
}
void orc_set_inlier(void *hp, const float *in) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, memcpy(vol->inlier.data(), in, vol->inlier.size() * 4));
}

void orc_mesh(void *hp) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->mesh());
}

// Mesh dump, pool independent: vertices sorted by key as vkeys[4i] =
// (x, y, z, slot), vdata[8i] = pos, normal, radius, ref; triangles sorted as
// tris[7t] = (cube x, y, z, slot, vertex indices i0, i1, i2).
void orc_dump_mesh(void *hp, int maxv, int32_t *vkeys, float *vdata, int maxt, int32_t *tr, int *nv, int *ntr) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    std::vector<uint64_t> ks;
    ks.reserve(vol->verts.size());
    for (auto &kv : vol->verts) ks.push_back(kv.first);
    std::sort(ks.begin(), ks.end());
    std::unordered_map<uint64_t, int> idx;
    for (size_t i = 0; i < ks.size(); ++i) idx[ks[i]] = (int)i;
    *nv = (int)ks.size();
    for (int i = 0; i < (int)ks.size() && i < maxv && vkeys; ++i) {
      uint64_t k = ks[i];
      vkeys[4 * i] = sext20(k >> 42), vkeys[4 * i + 1] = sext20(k >> 22), vkeys[4 * i + 2] = sext20(k >> 2);
      vkeys[4 * i + 3] = (int)(k & 3);
      auto &vt = vol->verts[k];
      float *d = vdata + 8 * i;
      d[0] = (float)vt.pos[0], d[1] = (float)vt.pos[1], d[2] = (float)vt.pos[2];
      d[3] = (float)vt.normal[0], d[4] = (float)vt.normal[1], d[5] = (float)vt.normal[2];
      d[6] = (float)vt.radius, d[7] = (float)vt.ref;
    }
    std::vector<uint64_t> tk;
    for (auto &kv : vol->tris) tk.push_back(kv.first);
    std::sort(tk.begin(), tk.end());
    int t = 0;
    for (uint64_t k : tk) {
      Tris &T = vol->tris[k];
      for (int s = 0; s < T.n; ++s, ++t) {
        if (t >= maxt || !tr) continue;
        int32_t *o = tr + 7 * t;
        o[0] = sext20(k >> 42), o[1] = sext20(k >> 22), o[2] = sext20(k >> 2), o[3] = s;
        for (int q = 0; q < 3; ++q) {
          auto it = idx.find(T.v[s][q]);
          o[4 + q] = it == idx.end() ? -1 : it->second;
        }
      }
    }
    *ntr = t;
  });
}

// Load a mesh state (same layout as the dump); replaces the current one.
void orc_load_mesh(void *hp, int nv, const int32_t *vkeys, const float *vdata, int nt, const int32_t *tr) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    vol->verts.clear();
    vol->tris.clear();
    std::vector<uint64_t> ks(nv);
    for (int i = 0; i < nv; ++i) {
      uint64_t k = vkey(vkeys[4 * i], vkeys[4 * i + 1], vkeys[4 * i + 2], vkeys[4 * i + 3]);
      ks[i] = k;
      auto &vt = vol->verts[k];
      const float *d = vdata + 8 * i;
      vt.pos[0] = d[0], vt.pos[1] = d[1], vt.pos[2] = d[2];
      vt.normal[0] = d[3], vt.normal[1] = d[4], vt.normal[2] = d[5];
      vt.radius = d[6], vt.ref = (int)d[7];
    }
    for (int t = 0; t < nt; ++t) {
      const int32_t *o = tr + 7 * t;
      Tris &T = vol->tris[vkey(o[0], o[1], o[2], 0)];
      int s = o[3];
      for (int q = 0; q < 3; ++q) T.v[s][q] = ks[o[4 + q]];
      if (s + 1 > T.n) T.n = (uint8_t)(s + 1);
    }
  });
}

void orc_get_cubes(void *hp, int n, const int32_t *pos, uint8_t *out) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    for (int i = 0; i < n; ++i) {
      int id = vol->find(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      if (id < 0) memset(out + (size_t)i * kBV, 0, kBV);
      else memcpy(out + (size_t)i * kBV, vol->blocks[id]->cube, kBV);
    }
  });
}
void orc_set_cubes(void *hp, int n, const int32_t *pos, const uint8_t *in) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    for (int i = 0; i < n; ++i) {
      int id = vol->find(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      if (id >= 0) memcpy(vol->blocks[id]->cube, in + (size_t)i * kBV, kBV);
    }
  });
}

void orc_get_block_meta(void *hp, int n, const int32_t *pos, int32_t *life, int32_t *inner, int32_t *boundary,
                        uint8_t *flag) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    for (int i = 0; i < n; ++i) {
      int id = vol->find(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      if (id < 0) continue;
      auto *b = vol->blocks[id].get();
      if (life) life[i] = b->life;
      if (inner) inner[i] = b->inner;
      if (boundary) boundary[i] = b->boundary;
      if (flag) flag[i] = b->flag;
    }
  });
}
void orc_set_block_meta(void *hp, int n, const int32_t *pos, const int32_t *life, const int32_t *inner,
                        const int32_t *boundary) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    for (int i = 0; i < n; ++i) {
      int id = vol->find(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
      if (id < 0) continue;
      auto *b = vol->blocks[id].get();
      if (life) b->life = life[i];
      if (inner) b->inner = inner[i];
      if (boundary) b->boundary = boundary[i];
    }
  });
}

void orc_raycast(void *hp, const float *cTw, float *depth, float *vert, float *norm) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    using R = std::remove_reference<decltype(*vol)>::type;
    (void)sizeof(R);
    decltype(vol->cTw) m;
    for (int i = 0; i < 16; ++i) m.e[i] = cTw[i];
    vol->raycast(m, depth, vert, norm);
  });
}

void orc_raycast_backward(void *hp, const float *cTw, const float *dL_dD, const float *dL_dN, double *xi) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    decltype(vol->cTw) m;
    for (int i = 0; i < 16; ++i) m.e[i] = cTw[i];
    vol->raycast_backward(m, dL_dD, dL_dN, xi);
  });
}

// the gradient of the last backward, per block with any entry: positions and
// 512 values each (returns the count; fills at most max_n)
int orc_grad_blocks(void *hp, int max_n, int32_t *pos, double *out) {
  OHandle *h = (OHandle *)hp;
  int n = 0;
  DISPATCH(h, {
    std::vector<int> ids;
    for (auto &kv : vol->grad) ids.push_back(kv.first);
    std::sort(ids.begin(), ids.end());
    for (int id : ids) {
      if (n < max_n) {
        const auto *b = vol->blocks[id].get();
        if (pos) pos[3 * n] = b->x, pos[3 * n + 1] = b->y, pos[3 * n + 2] = b->z;
        if (out) memcpy(out + (size_t)n * 512, vol->grad[id].data(), sizeof(double) * 512);
      }
      ++n;
    }
  });
  return n;
}

void orc_trace(void *hp, const float *cTw, int32_t *out) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    decltype(vol->cTw) m;
    for (int i = 0; i < 16; ++i) m.e[i] = cTw[i];
    vol->trace_dump(m, out);
  });
}

void orc_debug_ray(void *hp, const float *cTw, int x, int y, double *out) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    decltype(vol->cTw) m;
    for (int i = 0; i < 16; ++i) m.e[i] = cTw[i];
    vol->debug_ray(m, x, y, out);
  });
}

void orc_gc_low_surfel(void *hp) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->gc_low_surfel());
}
void orc_gc_starve(void *hp) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->gc_starve());
}
void orc_gc_collect_garbage(void *hp) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->gc_collect_garbage());
}
int orc_gc_recycle(void *hp) {
  OHandle *h = (OHandle *)hp;
  int n = 0;
  DISPATCH(h, n = vol->gc_recycle());
  return n;
}

void orc_point_to_psdf(void *hp, const float *wTc, int fix_j, double *A, double *b, double *err, int *count) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    decltype(vol->wTc) m;
    for (int i = 0; i < 16; ++i) m.e[i] = wTc[i];
    vol->point_to_psdf(m, fix_j != 0, A, b, *err, *count);
  });
}

void orc_huber_init(void *hp) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->huber_init());
}
void orc_huber_iterate(void *hp, float lambda, float sigma, float tau, int iters, double *err) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    vol->huber_iterate(lambda, sigma, tau, iters);
    err[0] = vol->pd_err[0], err[1] = vol->pd_err[1];
  });
}

// the single-precision exp of the PSDF path (mh_exp.h), for its accuracy test
void orc_expf(int n, const float *x, float *out) {
  for (int i = 0; i < n; ++i) out[i] = mh_expf(x[i]);
}
// replace the current frame's preprocessed depth (after orc_frame_set), e.g.
// with the library's denoised frame, so later stages start from the same input
void orc_set_depth(void *hp, const float *d) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, std::copy(d, d + vol->depth.size(), vol->depth.begin()));
}
void orc_denoise_tv(void *hp, float lambda, int iters) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, vol->denoise_tv(lambda, iters));
}
void orc_get_depth(void *hp, float *out) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, memcpy(out, vol->depth.data(), vol->depth.size() * 4));
}

// One MainEngine frame (app/reconstruction.cc:82-100; main_engine.cc:100-192)
// with the optional TV pre-filter: Mapping, Meshing (+ low-surfel GC, recycle every
// 10 frames), raycast into the given buffers (may be NULL), simple-mode
// Recycle every 15 frames.
void orc_frame(void *hp, const float *depth, const float *wTc, int tv_iters, float tv_lambda, float *rdepth,
               float *rvert, float *rnorm) {
  OHandle *h = (OHandle *)hp;
  DISPATCH(h, {
    vol->frame_set(depth, wTc);
    if (tv_iters > 0) vol->denoise_tv(tv_lambda, tv_iters);
    vol->allocate();
    vol->collect_frustum();
    if (vol->p.enable_bayesian_update) {
      vol->predict_inlier();
      vol->integrate_psdf();
    } else {
      vol->integrate_simple();
    }
    vol->frames++;
    vol->mesh();
    vol->gc_low_surfel();
    if (vol->frames % 10 == 0) vol->gc_recycle();
    if (rdepth || rvert || rnorm) vol->raycast(vol->cTw, rdepth, rvert, rnorm);
    if (!vol->p.enable_bayesian_update && vol->frames % 15 == 14) {
      vol->gc_starve();
      vol->gc_collect_garbage();
      vol->gc_recycle();
    }
  });
}

}  // extern "C"
