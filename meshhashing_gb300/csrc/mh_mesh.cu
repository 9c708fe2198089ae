// mh_mesh.cu -- per-block marching cubes with shared, ref-counted vertices.
//
// Follows MarchingCubes (meshing/marching_cubes.cu:326-382) and its
// shared-vertex layout: the vertex on the edge (v, v + axis) lives in slot
// `axis` of voxel v's mesh unit (kEdgeOwnerCubeOffset, mc_tables.h:360-376);
// each cube keeps up to five triangle slots that are reused across frames;
// vertices carry reference counts and are freed when no triangle uses them.
//
// GB300 structure, per mesh call:
//   k_mc_cubes     one 512-thread CTA per candidate block (persistent grid);
//                  a block with no mesh page whose weight bound is below the
//                  MC gate (inv_sigma2 >= 1/voxel^2) has no valid cube and is
//                  skipped after one 4-byte read;
//                  the 9x9x9 corner tile (block + x/y/z halo) is staged in
//                  shared memory as valid/negative bits, after 7 neighbour
//                  lookups per block instead of 8 per cube; each cube gets its
//                  index and claims the vertices of its cut edges for this
//                  epoch (one atomicCAS on the owner's claim word); the first
//                  claimer appends (owner, slot) to a compact work list.
//   k_mc_vertices  one thread per claimed vertex: warp-aggregated pool pops,
//                  position (VertexIntersection, marching_cubes.cu:16-28)
//                  from the owner cube's view of the edge, radius and SDF
//                  gradient normal (marching_cubes.cu:49-71).  Each vertex is
//                  computed exactly once, so the result does not depend on
//                  which of the up to four sharing cubes ran last.
//   k_mc_triangles surfel counts and triangle slot reuse/allocation with
//                  warp-aggregated pops (TriangleExtractionKernel, :180-275).
//   k_mc_recycle_* surplus triangle slots and unreferenced vertices return to
//                  their pools (RecycleTrianglesKernel / RecycleVerticesKernel,
//                  :278-321); a page left with no vertex and no triangle is
//                  returned as well.
// Mesh units live in mesh pages: a block receives one when a cube in it has
// triangles or a cube claims a vertex it owns.  The triangle and recycle
// passes walk only the candidates that hold a page.
#include "mh_internal.cuh"
#include "mh_kernels.h"
#include "mh_batch.cuh"

#define MH_MC_TABLE_QUALIFIER __constant__
#include "mc_cases.inc"

// Corner i of the cube at voxel v sits at v + kCorner[i] (mc_tables.h:335-344).
__constant__ int kCorner[8][3] = {{0, 1, 1}, {1, 1, 1}, {1, 1, 0}, {0, 1, 0},
                                  {0, 0, 1}, {1, 0, 1}, {1, 0, 0}, {0, 0, 0}};
// Corners joined by edge e (mc_tables.h:376-390).
__constant__ int kEdgeEnds[12][2] = {{0, 1}, {1, 2}, {2, 3}, {3, 0}, {4, 5}, {5, 6},
                                     {6, 7}, {7, 4}, {4, 0}, {5, 1}, {6, 2}, {7, 3}};
// Owner of edge e: its lower endpoint's offset and the edge axis (= slot);
// equal to kEdgeOwnerCubeOffset (mc_tables.h:360-374).
__constant__ int kOwner[12][4] = {{0, 1, 1, 0}, {1, 1, 0, 2}, {0, 1, 0, 0}, {0, 1, 0, 2},
                                  {0, 0, 1, 0}, {1, 0, 0, 2}, {0, 0, 0, 0}, {0, 0, 0, 2},
                                  {0, 0, 1, 1}, {1, 0, 1, 1}, {1, 0, 0, 1}, {0, 0, 0, 1}};

__device__ __forceinline__ int case_tris(int c) { return (int)(kMcCases[c] & 0xF); }
__device__ __forceinline__ int case_edge(int c, int k) { return (int)((kMcCases[c] >> (4 + 4 * k)) & 0xF); }

// claim slot `slot` of claim word `cw` for `epoch`; true for the first claimer
__device__ __forceinline__ bool claim_slot(const Dev &d, uint32_t *cw, int slot, unsigned epoch) {
  const uint32_t tag = epoch << 3, bit = 1u << slot;
  uint32_t old = *reinterpret_cast<volatile uint32_t *>(cw);
  for (int it = 0; it < 4096; ++it) {
    const bool same = (old & ~7u) == tag;
    if (same && (old & bit)) return false;
    const uint32_t nw = same ? (old | bit) : (tag | bit);
    const uint32_t prev = atomicCAS(cw, old, nw);
    if (prev == old) return true;
    old = prev;
  }
  set_error(d, MH_ERR_TIMEOUT);
  return false;
}

__device__ __forceinline__ void mc_begin_body(const Dev &d) {
  d.ctr->epoch += 1;
  d.ctr->vwork_count = 0;
  d.ctr->mesh_list_count = 0;
  d.ctr->cube_list_count = 0;
}
__global__ void k_mc_begin(Dev d) { mc_begin_body(d); }
// one thread per scene (the body is a single-thread step)
__global__ void k_mc_begin_b(const Scene *t, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && t[i].active) mc_begin_body(t[i].d);
}

// Candidates the cube pass must tile: a block holding a mesh page, or one
// whose weight bound reaches the MC gate (otherwise no cube in it is valid).
// One thread per candidate, warp-ballot compaction.
__device__ __forceinline__ void mc_select_body(const Dev &d) {
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  const float lim = 1.0f / d.p.voxel_size;
  const float lim2 = lim * lim;
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    int4 cb = make_int4(0, 0, 0, -1);
    bool keep = false;
    if (i < n) {
      cb = d.cand[i];
      keep = cb.w >= 0 && (d.page_of[cb.w] >= 0 || !(d.wmax[cb.w] < lim2));
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    int slot = 0;
    if (lane_id() == 0 && m) slot = atomicAdd(&d.ctr->cube_list_count, __popc(m));
    slot = __shfl_sync(0xffffffffu, slot, 0);
    if (keep) d.cube_list[slot + __popc(m & lanemask_lt())] = cb;
  }
}
__global__ void __launch_bounds__(256) k_mc_select(Dev d) { mc_select_body(d); }
__global__ void __launch_bounds__(256) k_mc_select_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { mc_select_body(c.d); });
}
__device__ __forceinline__ void mc_end_body(const Dev &d) {
  d.ctr->mesh_passes += 1;
  d.ctr->cand_sum += (unsigned long long)d.ctr->cand_count;
  d.ctr->vwork_sum += (unsigned long long)min(d.ctr->vwork_count, d.vwork_capacity);
  d.ctr->mesh_list_sum += (unsigned long long)d.ctr->mesh_list_count;
}
__global__ void k_mc_end(Dev d) { mc_end_body(d); }
// one thread per scene (the body is a single-thread step)
__global__ void k_mc_end_b(const Scene *t, int n) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n && t[i].active) mc_end_body(t[i].d);
}

// ------------------------------------------------------------------ pass 1
__device__ __forceinline__ void mc_cubes_body(const Dev &d) {
  __shared__ uint8_t tile[729];
  __shared__ int nb[8];
  __shared__ int own_page;
  const int tid = threadIdx.x;
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cube_list_count);
  const unsigned epoch = *reinterpret_cast<volatile unsigned *>(&d.ctr->epoch);
  const float lim = 1.0f / d.p.voxel_size;
  const float lim2 = lim * lim;
  const int x = tid & 7, y = (tid >> 3) & 7, z = tid >> 6;
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int4 cb = d.cube_list[c];
    if (tid < 8) {
      const int dx = tid & 1, dy = (tid >> 1) & 1, dz = tid >> 2;
      nb[tid] = tid == 0 ? cb.w : hash_find(d, cb.x + dx, cb.y + dy, cb.z + dz);
      if (tid == 0) atomicAdd(&d.ctr->cube_blocks_sum, 1ull);
    }
    __syncthreads();
    for (int e = tid; e < 729; e += 512) {
      const int tx = e % 9, ty = (e / 9) % 9, tz = e / 81;
      const int ptr = nb[(tx >> 3) + 2 * (ty >> 3) + 4 * (tz >> 3)];
      uint8_t f = 0;
      if (ptr >= 0) {
        const size_t gi = (size_t)ptr * MH_BLOCK_VOXELS + (tx & 7) + 8 * (ty & 7) + 64 * (tz & 7);
        const float s = d.sdf[gi], w = d.w[gi], a = d.a[gi], b = d.b[gi];
        const float rho = a / (a + b);
        const bool ok = !(fabsf(s) > 0.20f) && !(rho < 0.1f || w < lim2);
        f = (ok ? 1 : 0) | (s < 0.0f ? 2 : 0);
      }
      tile[e] = f;
    }
    __syncthreads();
    int cube = 0;
    bool valid = true;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const uint8_t f = tile[(x + kCorner[k][0]) + 9 * (y + kCorner[k][1]) + 81 * (z + kCorner[k][2])];
      valid &= (f & 1) != 0;
      cube |= ((f >> 1) & 1) << k;
    }
    if (!valid) cube = 0;
    const bool surf = cube != 0 && cube != 255;
    const int any_surf = __syncthreads_or(surf);
    if (tid == 0) own_page = any_surf ? ensure_page(d, cb.w) : d.page_of[cb.w];
    __syncthreads();
    const int pg = own_page;
    if (pg >= 0) d.cube[(size_t)pg * MH_BLOCK_VOXELS + tid] = (uint8_t)cube;
    if (surf && pg >= 0) {
#pragma unroll 1
      for (int e = 0; e < 12; ++e) {
        if (((cube >> kEdgeEnds[e][0]) & 1) == ((cube >> kEdgeEnds[e][1]) & 1)) continue;
        const int ox = x + kOwner[e][0], oy = y + kOwner[e][1], oz = z + kOwner[e][2];
        const int optr = nb[(ox >> 3) + 2 * (oy >> 3) + 4 * (oz >> 3)];
        if (optr < 0) continue;
        const int opg = ensure_page(d, optr);
        if (opg < 0) continue;
        const int oli = (ox & 7) + 8 * (oy & 7) + 64 * (oz & 7);
        const int slot = kOwner[e][3];
        if (claim_slot(d, d.claim + (size_t)opg * MH_BLOCK_VOXELS + oli, slot, epoch)) {
          const int wi = atomicAdd(&d.ctr->vwork_count, 1);
          if (wi < d.vwork_capacity) d.vwork[wi] = make_int4(opg, oli, slot, optr);
          else set_error(d, MH_ERR_CAPACITY);
        }
      }
    }
    __syncthreads();
  }
}
__global__ void __launch_bounds__(512) k_mc_cubes(Dev d) { mc_cubes_body(d); }
__global__ void __launch_bounds__(512) k_mc_cubes_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { mc_cubes_body(c.d); });
}

// candidates holding a page after pass 1; the others get zero surfel counts
__device__ __forceinline__ void mc_list_body(const Dev &d) {
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->cand_count);
  const int stride = gridDim.x * blockDim.x;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    int ptr = -1;
    bool keep = false;
    if (i < n) {
      ptr = d.cand[i].w;
      if (ptr >= 0) {
        keep = d.page_of[ptr] >= 0;
        if (!keep) d.inner[ptr] = d.boundary[ptr] = 0;
      }
    }
    const unsigned m = __ballot_sync(0xffffffffu, keep);
    int slot = 0;
    if (lane_id() == 0 && m) slot = atomicAdd(&d.ctr->mesh_list_count, __popc(m));
    slot = __shfl_sync(0xffffffffu, slot, 0);
    if (keep) d.mesh_list[slot + __popc(m & lanemask_lt())] = ptr;
  }
}
__global__ void __launch_bounds__(256) k_mc_list(Dev d) { mc_list_body(d); }
__global__ void __launch_bounds__(256) k_mc_list_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { mc_list_body(c.d); });
}

// ------------------------------------------------------------------ vertices
__device__ __forceinline__ void mc_vertices_body(const Dev &d) {
  const int n = min(*reinterpret_cast<volatile int *>(&d.ctr->vwork_count), d.vwork_capacity);
  const int stride = gridDim.x * blockDim.x;
  const float vs = d.p.voxel_size;
  for (int base = blockIdx.x * blockDim.x; base < n; base += stride) {
    const int i = base + threadIdx.x;
    const bool live = i < n;
    int4 wk = make_int4(0, 0, 0, 0);
    int *slotp = nullptr;
    int vp = -1;
    if (live) {
      wk = d.vwork[i];
      slotp = d.vtx_slot + ((size_t)wk.x * MH_BLOCK_VOXELS + wk.y) * 3 + wk.z;
      vp = *slotp;
    }
    const int fresh = warp_pop(d, &d.ctr->vtx_top, d.vtx_heap, live && vp < 0);
    if (!live) continue;
    const int blk = wk.w;
    if (vp < 0) {
      if (fresh < 0) continue;
      vp = fresh;
      *slotp = vp;
      atomicAdd(d.nvtx + blk, 1);
    }
    const int4 bp = d.block_pos[blk];
    const int slot = wk.z;
    const int v0x = bp.x * MH_BLOCK_SIDE + (wk.y & 7), v0y = bp.y * MH_BLOCK_SIDE + ((wk.y >> 3) & 7),
              v0z = bp.z * MH_BLOCK_SIDE + (wk.y >> 6);
    const int v1x = v0x + (slot == 0), v1y = v0y + (slot == 1), v1z = v0z + (slot == 2);
    BlockCache bc;
    bc.init();
    const float d0 = d.sdf[(size_t)blk * MH_BLOCK_VOXELS + wk.y];
    const int b1x = vox2blk(v1x), b1y = vox2blk(v1y), b1z = vox2blk(v1z);
    const int p1 = bc.get(d, b1x, b1y, b1z);
    const float d1 = p1 >= 0 ? d.sdf[(size_t)p1 * MH_BLOCK_VOXELS + (v1x - b1x * 8) + 8 * (v1y - b1y * 8) +
                                     64 * (v1z - b1z * 8)]
                             : 0.0f;
    // owner cube's endpoint order: x edge (v+x, v), y edge (v, v+y), z edge (v, v+z)
    const F3 P = f3((float)v0x * vs, (float)v0y * vs, (float)v0z * vs);
    const F3 Q = f3(P.x + vs * (float)(slot == 0), P.y + vs * (float)(slot == 1), P.z + vs * (float)(slot == 2));
    F3 p1w, p2w;
    float e1, e2;
    if (slot == 0) {
      p1w = Q, p2w = P, e1 = d1, e2 = d0;
    } else {
      p1w = P, p2w = Q, e1 = d0, e2 = d1;
    }
    F3 pos;
    if ((double)fabsf(e1) < 0.008) {
      pos = p1w;
    } else if ((double)fabsf(e2) < 0.008) {
      pos = p2w;
    } else {
      const float mu = (0.0f - e1) / (e2 - e1);
      pos = f3(p1w.x + mu * (p2w.x - p1w.x), p1w.y + mu * (p2w.y - p1w.y), p1w.z + mu * (p2w.z - p1w.z));
    }
    float s, rad, radius = 0.0f;
    if (spatial_sample<true>(d, bc, pos, s, rad)) {
      const float is2 = 1.0f / (rad * rad);
      radius = sqrtf(1.0f / is2);
    }
    F3 g;
    const bool ok = spatial_gradient(d, bc, pos, g);
    const float l = sqrtf(dot3(g, g));
    F3 nrm = f3(0.0f, 0.0f, 0.0f);
    if (ok && l > 0.0f) nrm = f3(g.x / l, g.y / l, g.z / l);
    Vertex *vt = d.vtx + vp;
    float4 *v4 = reinterpret_cast<float4 *>(vt);
    const int ref = vt->ref_count;
    v4[0] = make_float4(pos.x, pos.y, pos.z, nrm.x);
    v4[1] = make_float4(nrm.y, nrm.z, radius, __int_as_float(ref));
  }
}
__global__ void __launch_bounds__(128) k_mc_vertices(Dev d) { mc_vertices_body(d); }
__global__ void __launch_bounds__(128) k_mc_vertices_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { mc_vertices_body(c.d); });
}

// ------------------------------------------------------------------ pass 2
__device__ __forceinline__ void mc_triangles_body(const Dev &d) {
  __shared__ int nbp[8];
  __shared__ int cnt[2];
  const int tid = threadIdx.x;
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->mesh_list_count);
  const int x = tid & 7, y = (tid >> 3) & 7, z = tid >> 6;
  const bool inner = x >= 1 && y >= 1 && z >= 1 && x < 7 && y < 7 && z < 7;
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int blk = d.mesh_list[c];
    const int4 bp = d.block_pos[blk];
    if (tid < 8) {
      const int dx = tid & 1, dy = (tid >> 1) & 1, dz = tid >> 2;
      const int q = tid == 0 ? blk : hash_find(d, bp.x + dx, bp.y + dy, bp.z + dz);
      nbp[tid] = q >= 0 ? d.page_of[q] : -1;
    }
    if (tid < 2) cnt[tid] = 0;
    __syncthreads();
    const int pg = nbp[0];
    const size_t vi = (size_t)pg * MH_BLOCK_VOXELS + tid;
    // surfel counts (marching_cubes.cu:191-212)
    const int *vs = d.vtx_slot + vi * 3;
    const int here = (vs[0] >= 0) + (vs[1] >= 0) + (vs[2] >= 0);
    const int wsum = __reduce_add_sync(0xffffffffu, inner ? here : 0);
    const int bsum = __reduce_add_sync(0xffffffffu, inner ? 0 : here);
    if ((tid & 31) == 0) {
      if (wsum) atomicAdd(&cnt[0], wsum);
      if (bsum) atomicAdd(&cnt[1], bsum);
    }
    const int cube = d.cube[vi];
    const int ntri = (cube == 0 || cube == 255) ? 0 : case_tris(cube);
    int *ts = d.tri_slot + vi * 5;
#pragma unroll 1
    for (int t = 0; t < 5; ++t) {
      const bool need = t < ntri;
      const int old = need ? ts[t] : 0;
      const int fresh = warp_pop(d, &d.ctr->tri_top, d.tri_heap, need && old < 0);
      if (!need) continue;
      int vids[3];
      bool okv = true;
#pragma unroll
      for (int q = 0; q < 3; ++q) {
        const int e = case_edge(cube, 3 * t + q);
        const int ox = x + kOwner[e][0], oy = y + kOwner[e][1], oz = z + kOwner[e][2];
        const int opg = nbp[(ox >> 3) + 2 * (oy >> 3) + 4 * (oz >> 3)];
        const int oli = (ox & 7) + 8 * (oy & 7) + 64 * (oz & 7);
        vids[q] = opg >= 0 ? d.vtx_slot[((size_t)opg * MH_BLOCK_VOXELS + oli) * 3 + kOwner[e][3]] : -1;
        okv &= vids[q] >= 0;
      }
      int tp = old;
      if (old >= 0) {
        const int4 ot = d.tri[old];
        atomicSub(&d.vtx[ot.x].ref_count, 1);
        atomicSub(&d.vtx[ot.y].ref_count, 1);
        atomicSub(&d.vtx[ot.z].ref_count, 1);
      } else {
        tp = fresh;
        if (tp < 0) continue;
        ts[t] = tp;
      }
      if (!okv) {
        // a pool ran dry earlier in this pass; keep the slot on the reserved vertex 0
        set_error(d, MH_ERR_CAPACITY);
        d.tri[tp] = make_int4(0, 0, 0, 0);
        atomicAdd(&d.vtx[0].ref_count, 3);
        continue;
      }
      d.tri[tp] = make_int4(vids[0], vids[1], vids[2], 0);
      atomicAdd(&d.vtx[vids[0]].ref_count, 1);
      atomicAdd(&d.vtx[vids[1]].ref_count, 1);
      atomicAdd(&d.vtx[vids[2]].ref_count, 1);
    }
    __syncthreads();
    if (tid == 0) {
      d.inner[blk] = cnt[0];
      d.boundary[blk] = cnt[1];
    }
    __syncthreads();
  }
}
__global__ void __launch_bounds__(512) k_mc_triangles(Dev d) { mc_triangles_body(d); }
__global__ void __launch_bounds__(512) k_mc_triangles_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { mc_triangles_body(c.d); });
}

// ------------------------------------------------------------------ recycle
__device__ __forceinline__ void mc_recycle_tri_body(const Dev &d) {
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->mesh_list_count);
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int pg = d.page_of[d.mesh_list[c]];
    for (int v = threadIdx.x; v < MH_BLOCK_VOXELS; v += blockDim.x) {
      const size_t vi = (size_t)pg * MH_BLOCK_VOXELS + v;
      const int cube = d.cube[vi];
      const int ntri = (cube == 0 || cube == 255) ? 0 : case_tris(cube);
      int *ts = d.tri_slot + vi * 5;
      for (int t = ntri; t < 5; ++t) {
        const int tp = ts[t];
        if (tp < 0) continue;
        const int4 ot = d.tri[tp];
        atomicSub(&d.vtx[ot.x].ref_count, 1);
        atomicSub(&d.vtx[ot.y].ref_count, 1);
        atomicSub(&d.vtx[ot.z].ref_count, 1);
        d.tri[tp] = make_int4(-1, -1, -1, 0);
        stack_push(&d.ctr->tri_top, d.tri_heap, tp);
        ts[t] = MH_FREE_PTR;
      }
    }
  }
}
__global__ void __launch_bounds__(128) k_mc_recycle_tri(Dev d) { mc_recycle_tri_body(d); }
__global__ void __launch_bounds__(128) k_mc_recycle_tri_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { mc_recycle_tri_body(c.d); });
}

__device__ __forceinline__ void mc_recycle_vtx_body(const Dev &d) {
  __shared__ int live;
  const int n = *reinterpret_cast<volatile int *>(&d.ctr->mesh_list_count);
  for (int c = blockIdx.x; c < n; c += gridDim.x) {
    const int blk = d.mesh_list[c];
    const int pg = d.page_of[blk];
    if (threadIdx.x == 0) live = 0;
    __syncthreads();
    int freed = 0, used = 0;
    for (int v = threadIdx.x; v < MH_BLOCK_VOXELS * 3; v += blockDim.x) {
      int *sp = d.vtx_slot + (size_t)pg * MH_BLOCK_VOXELS * 3 + v;
      const int vp = *sp;
      if (vp < 0) continue;
      if (d.vtx[vp].ref_count != 0) {
        ++used;
        continue;
      }
      float4 *v4 = reinterpret_cast<float4 *>(d.vtx + vp);
      v4[0] = make_float4(0.f, 0.f, 0.f, 0.f);
      v4[1] = make_float4(0.f, 0.f, 0.f, 0.f);
      stack_push(&d.ctr->vtx_top, d.vtx_heap, vp);
      *sp = MH_FREE_PTR;
      ++freed;
    }
    for (int v = threadIdx.x; v < MH_BLOCK_VOXELS * 5; v += blockDim.x)
      used += d.tri_slot[(size_t)pg * MH_BLOCK_VOXELS * 5 + v] >= 0;
    if (freed) atomicSub(d.nvtx + blk, freed);
    if (used) atomicAdd(&live, used);
    __syncthreads();
    const bool empty = live == 0;
    __syncthreads();
    if (empty) release_page_cta(d, blk, pg);
    __syncthreads();
  }
}
__global__ void __launch_bounds__(128) k_mc_recycle_vtx(Dev d) { mc_recycle_vtx_body(d); }
__global__ void __launch_bounds__(128) k_mc_recycle_vtx_b(const Scene *t, int n) {
  each_scene(t, n, [&](const Scene &c) { mc_recycle_vtx_body(c.d); });
}

int launch_mesh(const Dev &d, cudaStream_t s) {
  const int sms = mh_sm_count();
  k_mc_begin<<<1, 1, 0, s>>>(d);
  k_mc_select<<<sms * 4, 256, 0, s>>>(d);
  k_mc_cubes<<<sms * 2, 512, 0, s>>>(d);
  k_mc_list<<<sms * 4, 256, 0, s>>>(d);
  k_mc_vertices<<<sms * 8, 128, 0, s>>>(d);
  k_mc_triangles<<<sms * 2, 512, 0, s>>>(d);
  k_mc_recycle_tri<<<sms * 8, 128, 0, s>>>(d);
  k_mc_recycle_vtx<<<sms * 8, 128, 0, s>>>(d);
  k_mc_end<<<1, 1, 0, s>>>(d);
  mh_count_launches(9);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}

int launch_batch_mesh(const Scene *t, int n, cudaStream_t s) {
  const int sms = mh_sm_count();
  k_mc_begin_b<<<(n + 63) / 64, 64, 0, s>>>(t, n);
  k_mc_select_b<<<sms * 4, 256, 0, s>>>(t, n);
  k_mc_cubes_b<<<sms * 2, 512, 0, s>>>(t, n);
  k_mc_list_b<<<sms * 4, 256, 0, s>>>(t, n);
  k_mc_vertices_b<<<sms * 8, 128, 0, s>>>(t, n);
  k_mc_triangles_b<<<sms * 2, 512, 0, s>>>(t, n);
  k_mc_recycle_tri_b<<<sms * 8, 128, 0, s>>>(t, n);
  k_mc_recycle_vtx_b<<<sms * 8, 128, 0, s>>>(t, n);
  k_mc_end_b<<<(n + 63) / 64, 64, 0, s>>>(t, n);
  mh_count_launches(9);
  return cudaGetLastError() == cudaSuccess ? MH_OK : MH_ERR_CUDA;
}
