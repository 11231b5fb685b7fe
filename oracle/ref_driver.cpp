/*
 * ref_driver.cpp -- runs libmat's own per-(tet, site) clipping kernel,
 * clipped_voro_cell_test_GPU_param_tet (src/rpd3d/convex_cell.cu:1166-1337),
 * on the CPU, one "GPU thread" at a time, and writes the surviving cells in
 * the packed record layout of rpd_oracle.h (topology sections only; the FP64
 * coordinate section is zero).  Test infrastructure: built by oracle/build.py
 * into oracle/_ref/ when the reference sources are present; used only to pin
 * the oracle.
 *
 * The reference sources are compiled in place (include path), never copied.
 * The inputs follow the reference's own layouts: SoA vertices / tets / sites,
 * the dense triangular e_adjs table (io.cxx:264-281), site_knn with
 * (site_k + 1) rows (triangulation.cxx:324-352) and tet_knn with tet_k rows
 * (voronoi.cu:306-317).
 */
#include "convex_cell.cu"

#include <cstring>
#include <thread>
#include <vector>

#include "../rpd_oracle.h"

namespace {
size_t al16(size_t x) { return (x + 15) & ~(size_t)15; }

/* the packed payload size of rpd_oracle.h, restated so this library stays
 * independent of the oracle */
size_t payload_bytes(int nb_v, int nb_p, int nb_e) {
  return (size_t)16 * nb_p + al16((size_t)8 * nb_p) + al16((size_t)4 * nb_v) +
         al16((size_t)4 * nb_e) + al16((size_t)nb_p) + al16((size_t)24 * nb_v);
}

void pack(const ConvexCellTransfer& c, uint8_t* out) {
  int np = c.nb_p, nv = c.nb_v, ne = c.nb_e;
  uint8_t* p = out;
  for (int i = 0; i < np; ++i) {
    float f[4] = {c.clip_data_trans[i].x, c.clip_data_trans[i].y,
                  c.clip_data_trans[i].z, c.clip_data_trans[i].w};
    std::memcpy(p + 16 * i, f, 16);
  }
  p += 16 * np;
  std::memset(p, 0, al16(8 * np));
  for (int i = 0; i < np; ++i) {
    int32_t v[2] = {c.clip_id2_data_trans[i].x, c.clip_id2_data_trans[i].y};
    std::memcpy(p + 8 * i, v, 8);
  }
  p += al16(8 * np);
  std::memset(p, 0, al16(4 * nv));
  for (int i = 0; i < nv; ++i) {
    p[4 * i + 0] = c.ver_data_trans[i].x;
    p[4 * i + 1] = c.ver_data_trans[i].y;
    p[4 * i + 2] = c.ver_data_trans[i].z;
    p[4 * i + 3] = c.ver_data_trans[i].w;
  }
  p += al16(4 * nv);
  std::memset(p, 0, al16(4 * ne));
  for (int i = 0; i < ne; ++i) {
    p[4 * i + 0] = c.edge_data[i].x;
    p[4 * i + 1] = c.edge_data[i].y;
    p[4 * i + 2] = c.edge_data[i].z;
  }
  p += al16(4 * ne);
  std::memset(p, 0, al16(np));
  for (int i = 0; i < np; ++i) p[i] = (uint8_t)c.clip_data_trans[i].h;
  p += al16(np);
  std::memset(p, 0, al16(24 * nv));
}
}  // namespace

extern "C" int64_t ref_clip_cells(
    int n_vert, const float* vert_soa, int n_tet, const int* idx_soa,
    const int* v_adjs, const int* e_adjs, const int* f_adjs, const int* f_ids,
    int n_site, const float* site_soa, const float* site_w,
    const unsigned* site_flags, const int* site_knn, int site_k,
    const int* tet_knn, int tet_k, orc_cell_header* headers,
    int32_t* thread_ids, uint8_t* payload, int64_t payload_capacity,
    int n_threads) {
  const int64_t n_slots = (int64_t)n_tet * tet_k;
  std::vector<int64_t> slot_pair(n_slots, -1);
  int64_t n_pairs = 0;
  for (int t = 0; t < n_tet; ++t)
    for (int s = 0; s < tet_k; ++s)
      if (tet_knn[(int64_t)s * n_tet + t] >= 0)
        slot_pair[(int64_t)t * tet_k + s] = n_pairs++;

  std::vector<int> status(n_slots, (int)early_return);
  std::vector<std::vector<uint8_t>> blobs(n_slots);
  std::vector<float> bary(3 * (size_t)n_site, 0.f), vol(n_site, 0.f);

  if (n_threads < 1) n_threads = 1;
  std::vector<std::thread> pool;
  for (int w = 0; w < n_threads; ++w) {
    pool.emplace_back([&, w]() {
      ConvexCellTransfer* tr = new ConvexCellTransfer();
      Status st;
      for (int64_t th = w; th < n_slots; th += n_threads) {
        if (slot_pair[th] < 0) continue;
        blockIdx.x = (unsigned)th;
        blockDim.x = 1;
        threadIdx.x = 0;
        tr->status = early_return;
        st = success;
        /* the kernel indexes its outputs by the global thread id */
        ConvexCellTransfer* cells_base = tr - th;
        Status* stat_base = &st - th;
        clipped_voro_cell_test_GPU_param_tet(
            site_soa, n_site, (size_t)n_site, site_w, site_flags, site_knn,
            (size_t)n_site, site_k, vert_soa, n_vert, (size_t)n_vert, idx_soa,
            n_tet, (size_t)n_tet, v_adjs, e_adjs, f_adjs, f_ids, tet_knn,
            (size_t)n_tet, tet_k, stat_base, nullptr, cells_base, bary.data(),
            (size_t)n_site, vol.data());
        if (tr->status == success) {
          status[th] = (int)success;
          size_t need = payload_bytes(tr->nb_v, tr->nb_p, tr->nb_e);
          blobs[th].resize(need);
          pack(*tr, blobs[th].data());
          headers[slot_pair[th]].nb_v = tr->nb_v;
          headers[slot_pair[th]].nb_p = tr->nb_p;
          headers[slot_pair[th]].nb_e = tr->nb_e;
        } else {
          /* the kernel's gpu_stat keeps the failure reason; a return
           * without a failure (seed not flagged) stays early_return */
          status[th] = st == success ? (int)early_return : (int)st;
        }
      }
      delete tr;
    });
  }
  for (auto& th : pool) th.join();

  int64_t off = 0;
  for (int64_t th = 0; th < n_slots; ++th) {
    int64_t q = slot_pair[th];
    if (q < 0) continue;
    orc_cell_header& h = headers[q];
    h.tet_id = (int32_t)(th / tet_k);
    h.site_id = tet_knn[(th % tet_k) * n_tet + th / tet_k];
    h.status = status[th];
    h.flags = 0;
    h.volume = 0.0;
    h.offset = (uint64_t)off;
    if (thread_ids) thread_ids[q] = (int32_t)th;
    if (status[th] == (int)success) {
      if (off + (int64_t)blobs[th].size() <= payload_capacity)
        std::memcpy(payload + off, blobs[th].data(), blobs[th].size());
      off += (int64_t)blobs[th].size();
    } else {
      h.nb_v = h.nb_p = h.nb_e = 0;
    }
  }
  return off <= payload_capacity ? off : -1;
}
