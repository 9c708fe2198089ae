// mh_io.cu -- block checkpoint / resume.
//
// The reference's logging engine (engine/logging_engine.cc:101-233) records
// the allocated blocks (positions and voxel values) and rebuilds the hash
// table when it reads them back.  Same idea here, as one binary file:
//   header  "MHVOL01\0", u32 block count, u32 field count (2: sdf and weight,
//           4: also the PSDF a and b), f32 voxel size, f32 truncation
//           distance, f32 truncation scale
//   blocks  per block: i32 x, y, z, then 512 floats per field
// Save and load stream the blocks in chunks of at most kIoChunk blocks (the
// host buffers hold one chunk of the file's fields, 16 MB at 4 fields), so a
// small map needs small buffers.  Loading inserts the blocks into the hash
// (the same path as mh_load_blocks) and leaves the mesh to the next mesh
// pass.  A file whose field count, voxel size or truncation differs from the
// volume's is refused before anything is inserted.
#include <algorithm>
#include <cstdio>
#include <cstring>
#include <vector>

#include "mh_kernels.h"
#include "mh_volume.h"

extern "C" int mh_load_blocks(mh_volume *v, int n, const int32_t *pos, const float *sdf, const float *weight,
                              const float *a, const float *b);

namespace {
const char kMagic[8] = {'M', 'H', 'V', 'O', 'L', '0', '1', '\0'};
constexpr int kIoChunk = 1 << 11;
struct Header {
  char magic[8];
  uint32_t blocks, fields;
  float voxel_size, truncation, truncation_scale;
};
}  // namespace

extern "C" {

int mh_save_volume(mh_volume *v, const char *path) {
  if (!v || !path) return MH_ERR_INVALID;
  if (cudaDeviceSynchronize() != cudaSuccess) return MH_ERR_CUDA;
  Counters c;
  if (cudaMemcpy(&c, v->d.ctr, sizeof(c), cudaMemcpyDeviceToHost) != cudaSuccess) return MH_ERR_CUDA;
  const int hw = c.high_water;
  const int nf = v->hp.enable_bayesian_update ? 4 : 2;
  const float *fields[4] = {v->d.sdf, v->d.w, v->d.a, v->d.b};
  FILE *f = fopen(path, "wb");
  if (!f) return MH_ERR_INVALID;
  Header h;
  memcpy(h.magic, kMagic, 8);
  h.blocks = 0;
  h.fields = (uint32_t)nf;
  h.voxel_size = v->hp.voxel_size, h.truncation = v->hp.truncation_distance;
  h.truncation_scale = v->hp.truncation_distance_scale;
  bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
  const int chunk = std::max(1, std::min(kIoChunk, hw));
  std::vector<int4> bp(chunk);
  std::vector<float> rows((size_t)chunk * MH_BLOCK_VOXELS * nf);
  uint32_t written = 0;
  for (int base = 0; base < hw && ok; base += chunk) {
    const int n = std::min(chunk, hw - base);
    if (cudaMemcpy(bp.data(), v->d.block_pos + base, sizeof(int4) * n, cudaMemcpyDeviceToHost) != cudaSuccess) {
      ok = false;
      break;
    }
    for (int fi = 0; fi < nf && ok; ++fi)
      ok = cudaMemcpy(rows.data() + (size_t)fi * chunk * MH_BLOCK_VOXELS,
                      fields[fi] + (size_t)base * MH_BLOCK_VOXELS, sizeof(float) * MH_BLOCK_VOXELS * n,
                      cudaMemcpyDeviceToHost) == cudaSuccess;
    for (int i = 0; i < n && ok; ++i) {
      if (!bp[i].w) continue;
      const int32_t p3[3] = {bp[i].x, bp[i].y, bp[i].z};
      ok = fwrite(p3, sizeof(int32_t), 3, f) == 3;
      for (int fi = 0; fi < nf && ok; ++fi)
        ok = fwrite(rows.data() + ((size_t)fi * chunk + i) * MH_BLOCK_VOXELS, sizeof(float), MH_BLOCK_VOXELS,
                    f) == MH_BLOCK_VOXELS;
      ++written;
    }
  }
  if (ok) {
    h.blocks = written;
    ok = fseek(f, 0, SEEK_SET) == 0 && fwrite(&h, sizeof(h), 1, f) == 1;
  }
  ok = (fclose(f) == 0) && ok;
  return ok ? MH_OK : MH_ERR_INVALID;
}

int mh_load_volume(mh_volume *v, const char *path, int *n_blocks) {
  if (!v || !path) return MH_ERR_INVALID;
  FILE *f = fopen(path, "rb");
  if (!f) return MH_ERR_INVALID;
  Header h;
  // the file must hold the fields this volume's update keeps (2: sdf and
  // weight of the simple update, 4: also the PSDF a and b) and come from the
  // same voxel size and truncation
  const uint32_t want_fields = v->hp.enable_bayesian_update ? 4u : 2u;
  if (fread(&h, sizeof(h), 1, f) != 1 || memcmp(h.magic, kMagic, 8) != 0 || h.fields != want_fields ||
      h.voxel_size != v->hp.voxel_size || h.truncation != v->hp.truncation_distance ||
      h.truncation_scale != v->hp.truncation_distance_scale) {
    fclose(f);
    return MH_ERR_INVALID;
  }
  const int nf = (int)h.fields;
  const int chunk = (int)std::max<uint32_t>(1, std::min<uint32_t>(kIoChunk, h.blocks));
  std::vector<int32_t> pos((size_t)chunk * 3);
  std::vector<float> fld((size_t)chunk * MH_BLOCK_VOXELS * nf, 0.0f);
  std::vector<float> rec((size_t)MH_BLOCK_VOXELS * nf);
  int r = MH_OK;
  uint32_t done = 0;
  while (done < h.blocks && r == MH_OK) {
    const int n = (int)std::min<uint32_t>(chunk, h.blocks - done);
    for (int i = 0; i < n && r == MH_OK; ++i) {
      if (fread(&pos[3 * i], sizeof(int32_t), 3, f) != 3 || fread(rec.data(), sizeof(float), rec.size(), f) != rec.size()) {
        r = MH_ERR_INVALID;
        break;
      }
      for (int fi = 0; fi < nf; ++fi)
        memcpy(&fld[((size_t)fi * chunk + i) * MH_BLOCK_VOXELS], &rec[(size_t)fi * MH_BLOCK_VOXELS],
               sizeof(float) * MH_BLOCK_VOXELS);
    }
    if (r != MH_OK) break;
    const float *F[4] = {fld.data(), fld.data() + (size_t)chunk * MH_BLOCK_VOXELS,
                         nf == 4 ? fld.data() + (size_t)2 * chunk * MH_BLOCK_VOXELS : nullptr,
                         nf == 4 ? fld.data() + (size_t)3 * chunk * MH_BLOCK_VOXELS : nullptr};
    r = mh_load_blocks(v, n, pos.data(), F[0], F[1], F[2], F[3]);
    done += (uint32_t)n;
  }
  fclose(f);
  if (n_blocks) *n_blocks = (int)done;
  return r;
}

}  // extern "C"
