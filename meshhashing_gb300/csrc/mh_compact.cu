// mh_compact.cu -- dense copy of the mesh and its PLY export.
//
// CompressMesh (visualization/compress_mesh.cu:10-172) gathers the vertices
// referenced by live triangles into a dense array and remaps the triangles;
// its per-CTA atomics make the output order vary from run to run.  Here the
// compaction is a stable prefix scan over the pools (vertex and triangle
// index order), so two calls on the same mesh give the same arrays:
//   1. mark every vertex referenced by a live triangle (all three vertex
//      indices > 0: index 0 is never handed out, and freed triangles are
//      marked -1);
//   2. per chunk of 1024 pool entries, count the kept ones; one CTA scans the
//      chunk counts; each chunk then places its entries with a ballot scan;
//   3. vertices go first and leave their new index in the mark array, which
//      the triangle pass reads to remap.
// The PLY writer (io/mesh_writer.cc:14-150 writes the reference's meshes) is
// binary little-endian: float x y z nx ny nz per vertex, one uchar-count
// int list per face.
#include <algorithm>
#include <cstdio>
#include <vector>

#include "mh_kernels.h"
#include "mh_volume.h"

namespace {

constexpr int kChunk = 1024;  // entries per chunk (256 threads x 4)

__device__ __forceinline__ bool tri_live(const int4 t) { return t.x > 0 && t.y > 0 && t.z > 0; }

__global__ void k_mark_vertices(const int4 *tri, int n_tri, int *mark) {
  for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < n_tri; t += gridDim.x * blockDim.x) {
    const int4 q = tri[t];
    if (!tri_live(q)) continue;
    mark[q.x] = 1, mark[q.y] = 1, mark[q.z] = 1;
  }
}

// keep(i) for the two pools
struct KeepVertex {
  const int *mark;
  __device__ bool operator()(int i) const { return mark[i] != 0; }
};
struct KeepTriangle {
  const int4 *tri;
  __device__ bool operator()(int i) const { return tri_live(tri[i]); }
};

template <class K> __global__ void __launch_bounds__(256) k_chunk_count(K keep, int n, int *counts) {
  const int base = blockIdx.x * kChunk;
  int c = 0;
  for (int k = 0; k < 4; ++k) {
    const int i = base + k * 256 + threadIdx.x;
    c += (i < n && keep(i)) ? 1 : 0;
  }
  __shared__ int red[8];
  for (int o = 16; o; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = c;
  __syncthreads();
  if (threadIdx.x == 0) {
    int s = 0;
    for (int w = 0; w < 8; ++w) s += red[w];
    counts[blockIdx.x] = s;
  }
}

// exclusive scan of counts[0, n) in place, total in counts[n]; one CTA of 1024
__global__ void __launch_bounds__(1024) k_scan_counts(int *counts, int n) {
  __shared__ int buf[1024];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < n; base += 1024) {
    const int i = base + threadIdx.x;
    const int v = i < n ? counts[i] : 0;
    buf[threadIdx.x] = v;
    __syncthreads();
    for (int o = 1; o < 1024; o <<= 1) {
      const int a = threadIdx.x >= o ? buf[threadIdx.x - o] : 0;
      __syncthreads();
      buf[threadIdx.x] += a;
      __syncthreads();
    }
    if (i < n) counts[i] = carry + buf[threadIdx.x] - v;
    __syncthreads();
    if (threadIdx.x == 1023) carry += buf[1023];
    __syncthreads();
  }
  if (threadIdx.x == 0) counts[n] = carry;
}

// position of entry i among the kept ones of its chunk, in index order
template <class K, class W>
__global__ void __launch_bounds__(256) k_chunk_place(K keep, int n, const int *offsets, W write) {
  __shared__ int warp_base[33];
  const int base = blockIdx.x * kChunk;
  int run = offsets[blockIdx.x];
  for (int k = 0; k < 4; ++k) {
    const int i = base + k * 256 + threadIdx.x;
    const bool kp = i < n && keep(i);
    const unsigned m = __ballot_sync(0xffffffffu, kp);
    if ((threadIdx.x & 31) == 0) warp_base[threadIdx.x >> 5] = __popc(m);
    __syncthreads();
    if (threadIdx.x == 0) {
      int s = run;
      for (int w = 0; w < 8; ++w) {
        const int c = warp_base[w];
        warp_base[w] = s;
        s += c;
      }
      warp_base[32] = s;
    }
    __syncthreads();
    if (kp) write(i, warp_base[threadIdx.x >> 5] + __popc(m & ((1u << (threadIdx.x & 31)) - 1u)));
    run = warp_base[32];
    __syncthreads();
  }
}

struct WriteVertex {
  const Vertex *vtx;
  int *remap;      // the mark array: becomes the new index
  float *pos, *nrm;
  __device__ void operator()(int i, int o) const {
    const Vertex v = vtx[i];
    pos[3 * o] = v.px, pos[3 * o + 1] = v.py, pos[3 * o + 2] = v.pz;
    nrm[3 * o] = v.nx, nrm[3 * o + 1] = v.ny, nrm[3 * o + 2] = v.nz;
    remap[i] = o;
  }
};
struct WriteTriangle {
  const int4 *tri;
  const int *remap;
  int *out;
  __device__ void operator()(int i, int o) const {
    const int4 t = tri[i];
    out[3 * o] = remap[t.x], out[3 * o + 1] = remap[t.y], out[3 * o + 2] = remap[t.z];
  }
};

template <class K> int count_kept(K keep, int n, int *counts, int chunks, cudaStream_t s) {
  k_chunk_count<<<chunks, 256, 0, s>>>(keep, n, counts);
  k_scan_counts<<<1, 1024, 0, s>>>(counts, chunks);
  mh_count_launches(2);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

}  // namespace

// Dense mesh into device arrays: pos3/nrm3 (>= max_vertex_count x 3 floats),
// tri3 (>= max_triangle_count x 3 ints); counts to host.
static int compact_device(mh_volume *v, float *pos3, float *nrm3, int *tri3, int &nv, int &nt, cudaStream_t s) {
  const int NV = (int)v->hp.max_vertex_count, NT = (int)v->hp.max_triangle_count;
  const int cv = (NV + kChunk - 1) / kChunk, ct = (NT + kChunk - 1) / kChunk;
  // scratch: mark/remap (NV) + vertex chunk counts (cv + 1) + triangle chunk counts (ct + 1)
  const size_t need = sizeof(int) * ((size_t)NV + cv + 1 + ct + 1);
  if (v->scratch_bytes < need) {
    if (v->scratch) cudaFree(v->scratch);
    v->scratch = nullptr;
    v->scratch_bytes = 0;
    if (cudaMalloc(&v->scratch, need) != cudaSuccess) return MH_ERR_NOMEM;
    v->scratch_bytes = need;
  }
  int *mark = v->scratch, *vcnt = mark + NV, *tcnt = vcnt + cv + 1;
  MH_CUDA_TRY(cudaMemsetAsync(mark, 0, sizeof(int) * NV, s));
  const int g = mh_sm_count() * 8;
  k_mark_vertices<<<g, 256, 0, s>>>(v->d.tri, NT, mark);
  mh_count_launches(1);
  KeepVertex kv{mark};
  KeepTriangle kt{v->d.tri};
  int r;
  if ((r = count_kept(kv, NV, vcnt, cv, s)) != MH_OK) return r;
  if ((r = count_kept(kt, NT, tcnt, ct, s)) != MH_OK) return r;
  // vertices first: their pass turns mark into the remap the triangles read
  k_chunk_place<<<cv, 256, 0, s>>>(kv, NV, vcnt, WriteVertex{v->d.vtx, mark, pos3, nrm3});
  k_chunk_place<<<ct, 256, 0, s>>>(kt, NT, tcnt, WriteTriangle{v->d.tri, mark, tri3});
  mh_count_launches(2);
  MH_CUDA_TRY(cudaGetLastError());
  int hv = 0, ht = 0;
  MH_CUDA_TRY(cudaMemcpyAsync(&hv, vcnt + cv, sizeof(int), cudaMemcpyDeviceToHost, s));
  MH_CUDA_TRY(cudaMemcpyAsync(&ht, tcnt + ct, sizeof(int), cudaMemcpyDeviceToHost, s));
  MH_CUDA_TRY(cudaStreamSynchronize(s));
  nv = hv, nt = ht;
  return MH_OK;
}

extern "C" {

int mh_mesh_compact(mh_volume *v, int max_vertices, float *positions3, float *normals3, int max_triangles,
                    int32_t *triangles3, int *n_vertices, int *n_triangles, int out_on_device, void *stream) {
  if (!v || max_vertices < 0 || max_triangles < 0) return MH_ERR_INVALID;
  cudaStream_t s = (cudaStream_t)stream;
  const size_t NV = v->hp.max_vertex_count, NT = v->hp.max_triangle_count;
  float *dp = nullptr;
  int *dt = nullptr;
  // device staging for the dense arrays (positions, normals: 3 floats per
  // vertex; triangles: 3 ints)
  if (cudaMalloc(&dp, sizeof(float) * 6 * NV) != cudaSuccess) return MH_ERR_NOMEM;
  if (cudaMalloc(&dt, sizeof(int) * 3 * NT) != cudaSuccess) {
    cudaFree(dp);
    return MH_ERR_NOMEM;
  }
  int nv = 0, nt = 0;
  int r = compact_device(v, dp, dp + 3 * NV, dt, nv, nt, s);
  if (r == MH_OK) {
    const cudaMemcpyKind k = out_on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
    const size_t cv = (size_t)std::min(nv, max_vertices), ctr = (size_t)std::min(nt, max_triangles);
    if ((positions3 && cv && cudaMemcpy(positions3, dp, sizeof(float) * 3 * cv, k) != cudaSuccess) ||
        (normals3 && cv && cudaMemcpy(normals3, dp + 3 * NV, sizeof(float) * 3 * cv, k) != cudaSuccess) ||
        (triangles3 && ctr && cudaMemcpy(triangles3, dt, sizeof(int) * 3 * ctr, k) != cudaSuccess))
      r = MH_ERR_CUDA;
  }
  cudaFree(dp);
  cudaFree(dt);
  if (n_vertices) *n_vertices = nv;
  if (n_triangles) *n_triangles = nt;
  return r;
}

static int fetch_compact(mh_volume *v, std::vector<float> &pos, std::vector<float> &nrm, std::vector<int32_t> &tri,
                         int &nv, int &nt) {
  nv = nt = 0;
  int r = mh_mesh_compact(v, 0, nullptr, nullptr, 0, nullptr, &nv, &nt, 0, nullptr);
  if (r != MH_OK) return r;
  pos.resize((size_t)nv * 3), nrm.resize((size_t)nv * 3), tri.resize((size_t)nt * 3);
  return mh_mesh_compact(v, nv, pos.data(), nrm.data(), nt, tri.data(), &nv, &nt, 0, nullptr);
}

int mh_write_ply(mh_volume *v, const char *path) {
  if (!v || !path) return MH_ERR_INVALID;
  std::vector<float> pos, nrm;
  std::vector<int32_t> tri;
  int nv, nt;
  int r = fetch_compact(v, pos, nrm, tri, nv, nt);
  if (r != MH_OK) return r;
  FILE *f = fopen(path, "wb");
  if (!f) return MH_ERR_INVALID;
  fprintf(f,
          "ply\nformat binary_little_endian 1.0\ncomment written by libmeshhash\nelement vertex %d\n"
          "property float x\nproperty float y\nproperty float z\nproperty float nx\nproperty float ny\n"
          "property float nz\nelement face %d\nproperty list uchar int vertex_indices\nend_header\n",
          nv, nt);
  bool ok = true;
  for (int i = 0; i < nv && ok; ++i) {
    float rec[6] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2], nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]};
    ok = fwrite(rec, sizeof(float), 6, f) == 6;
  }
  for (int i = 0; i < nt && ok; ++i) {
    const unsigned char three = 3;
    ok = fwrite(&three, 1, 1, f) == 1 && fwrite(&tri[3 * i], sizeof(int32_t), 3, f) == 3;
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? MH_OK : MH_ERR_INVALID;
}

// SaveObj (io/mesh_writer.cc:14-73): "v", then "vn" lines, then faces as
// 1-based "f a//a b//b c//c"; coordinates with 9 significant digits, which
// read back to the same floats.
int mh_write_obj(mh_volume *v, const char *path) {
  if (!v || !path) return MH_ERR_INVALID;
  std::vector<float> pos, nrm;
  std::vector<int32_t> tri;
  int nv, nt;
  int r = fetch_compact(v, pos, nrm, tri, nv, nt);
  if (r != MH_OK) return r;
  FILE *f = fopen(path, "w");
  if (!f) return MH_ERR_INVALID;
  bool ok = true;
  for (int i = 0; i < nv && ok; ++i)
    ok = fprintf(f, "v %.9g %.9g %.9g\n", pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]) > 0;
  for (int i = 0; i < nv && ok; ++i)
    ok = fprintf(f, "vn %.9g %.9g %.9g\n", nrm[3 * i], nrm[3 * i + 1], nrm[3 * i + 2]) > 0;
  for (int i = 0; i < nt && ok; ++i) {
    const int a = tri[3 * i] + 1, b = tri[3 * i + 1] + 1, c = tri[3 * i + 2] + 1;
    ok = fprintf(f, "f %d//%d %d//%d %d//%d\n", a, a, b, b, c, c) > 0;
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? MH_OK : MH_ERR_INVALID;
}

}  // extern "C"
