// rpd_batch.cpp -- many independent meshes in one run (rpd_batch_* of the C
// ABI).
//
// The meshes and their sites are concatenated into one context: vertex ids
// of the tets are offset by the mesh's first vertex, site ids (neighbour
// lists, pairs, plane ids on the device) by its first site.  The front end
// runs per mesh -- its own site grid and kNN, tet grids per radius class,
// candidate boxes and the pair search, each kernel told the mesh's site and
// tet bases -- and appends every mesh's pairs to one buffer.  The front end
// of all meshes is captured once into a CUDA graph (a few thousand small
// launches for hundreds of meshes) and replayed; it has no host
// synchronisation inside.  Then one CSR, ONE persistent clip launch over all
// meshes' pairs (uneven cells balance through its work counter), one
// epilogue and one compaction.  Cells of mesh m are a contiguous range of
// the compacted cells; rpd_batch_copy_mesh_cells returns them with the
// mesh's own tet and site ids, as a single-mesh run would.

#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "rpd_ctx.hpp"

namespace {

struct BatchMesh {
  int vert_base = 0, n_vert = 0, tet_base = 0, n_tet = 0, site_base = 0, n_site = 0;
  double mesh_lo[3], mesh_hi[3], site_lo[3], site_hi[3];
  float w_max = 0.f;
  int class_count[2] = {0, 0};
  double class_radius[2] = {0.0, 0.0};
  Grid site_grid;
  Grid tet_grid[2];
};

}  // namespace

// scratch of one front-end lane (a stream on which whole meshes run)
struct FrontLane {
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  DevBuf<int32_t> s_cell_count, s_cell_start, s_cell_fill, s_cell_items;
  DevBuf<int32_t> t_cell_of, t_cell_count, t_cell_start, t_cell_fill, t_cell_items;
  DevBuf<float> t_cell_rmax;
  DevBuf<int32_t> scan_tmp, pair_ntasks, pair_taskoff;
  DevBuf<unsigned long long> work;  // the pair kernel's task counter
  std::vector<int> meshes;           // meshes of this lane
};

constexpr int kFrontLanes = 8;

struct rpd_batch {
  rpd_ctx* ctx = nullptr;
  std::vector<BatchMesh> meshes;
  // host staging of the concatenated inputs
  std::vector<double> xyz, sites;
  std::vector<int32_t> tets, v_adjs, f_adjs, f_ids;
  std::vector<uint8_t> e_adj6, tet_class;
  std::vector<uint32_t> flags;
  bool uploaded = false;
  // front-end lanes: meshes spread over streams that run concurrently, each
  // with scratch sized for its largest mesh
  FrontLane lanes[kFrontLanes];
  cudaEvent_t fork = nullptr;
  DevBuf<int32_t> tet_base_dev;
  DevBuf<long long> mesh_first_dev;
  std::vector<long long> mesh_first;
  // the captured front end
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  int graph_launches = 0;
  bool use_graph = true;
  rpd_config captured_cfg;  // front-end fields the graph was recorded with
  std::string err;
};

namespace {

rpd_status bfail(rpd_batch* b, rpd_status s, const std::string& msg) {
  if (b) b->err = msg;
  return s;
}

#define BCK(expr, where)                                        \
  do {                                                          \
    cudaError_t _e = (expr);                                    \
    if (_e != cudaSuccess) {                                    \
      cudaGetLastError();                                       \
      return bfail(b, _e == cudaErrorMemoryAllocation ? RPD_ERR_OUT_OF_MEMORY : RPD_ERR_CUDA, \
                   std::string(where) + ": " + cudaGetErrorString(_e));                     \
    }                                                           \
  } while (0)

void drop_graph(rpd_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// uploads the concatenated inputs and sizes the front end's buffers
rpd_status upload(rpd_batch* b) {
  rpd_ctx* c = b->ctx;
  const int n_vert = (int)(b->xyz.size() / 3), n_tet = (int)(b->tets.size() / 4);
  const int n_site = (int)(b->sites.size() / 4);
  rpd_status s = rpd_set_mesh(c, b->xyz.data(), n_vert, b->tets.data(), n_tet, b->v_adjs.data(),
                              b->e_adj6.data(), b->f_adjs.data(), b->f_ids.data());
  if (s != RPD_OK) return bfail(b, s, rpd_last_error(c));
  s = rpd_set_sites(c, b->sites.data(), n_site, b->flags.data());
  if (s != RPD_OK) return bfail(b, s, rpd_last_error(c));
  cudaStream_t st = c->stream;
  // radius classes per mesh (the context's are over all tets)
  BCK(cudaMemcpy(c->tet_class.ptr, b->tet_class.data(), b->tet_class.size(), cudaMemcpyHostToDevice),
      "H2D classes");
  // each site's lists hold only its own mesh's sites (the exact-lists rounds
  // search one grid of every site)
  // (and, for that grid, each mesh moved to a slot of its own: meshes that
  // overlap in space would otherwise fill every grid cell with sites of the
  // others)
  {
    std::vector<int2> range((size_t)n_site);
    double ext[3] = {0, 0, 0};
    for (const BatchMesh& m : b->meshes)
      for (int a = 0; a < 3; ++a) ext[a] = std::max(ext[a], m.site_hi[a] - m.site_lo[a]);
    const int nm = (int)b->meshes.size();
    int side = 1;
    while ((long long)side * side * side < nm) ++side;
    double stride[3];
    for (int a = 0; a < 3; ++a) stride[a] = ext[a] * (1.0 + 1e-3) + 1e-6 * (ext[a] + 1.0);
    std::vector<float4> gpos((size_t)n_site);
    for (int mi = 0; mi < nm; ++mi) {
      const BatchMesh& m = b->meshes[(size_t)mi];
      const int slot[3] = {mi % side, (mi / side) % side, mi / (side * side)};
      double off[3];
      for (int a = 0; a < 3; ++a) off[a] = slot[a] * stride[a] - m.site_lo[a];
      for (int i = 0; i < m.n_site; ++i) {
        const size_t s = (size_t)(m.site_base + i);
        range[s] = make_int2(m.site_base, m.site_base + m.n_site);
        const double* x = &b->sites[4 * s];
        gpos[s] = make_float4((float)(x[0] + off[0]), (float)(x[1] + off[1]),
                              (float)(x[2] + off[2]), (float)x[3]);
      }
    }
    for (int a = 0; a < 3; ++a) {
      c->grid_lo[a] = 0.0;
      c->grid_hi[a] = stride[a] * (a == 0 ? side : (a == 1 ? std::min(side, (nm + side - 1) / side)
                                                          : (nm + side * side - 1) / (side * side)));
    }
    BCK(c->site_range.ensure((size_t)n_site), "alloc");
    BCK(cudaMemcpy(c->site_range.ptr, range.data(), sizeof(int2) * range.size(),
                   cudaMemcpyHostToDevice), "H2D ranges");
    BCK(c->site_gridpos.ensure((size_t)n_site), "alloc");
    BCK(cudaMemcpy(c->site_gridpos.ptr, gpos.data(), sizeof(float4) * gpos.size(),
                   cudaMemcpyHostToDevice), "H2D grid positions");
    c->has_site_range = true;
  }
  const int k = c->cfg.knn_k;
  c->k = k;
  BCK(c->nbr.ensure((size_t)n_site * k), "alloc");
  BCK(c->nbr_keys.ensure((size_t)n_site * k), "alloc");
  BCK(c->nbr_dist.ensure((size_t)n_site * k), "alloc");
  BCK(c->knn_status.ensure((size_t)n_site), "alloc");
  BCK(c->nbr_bound.ensure((size_t)n_site), "alloc");
  BCK(c->s_cell_of.ensure((size_t)n_site), "alloc");
  BCK(c->site_box.ensure((size_t)n_site * 2), "alloc");
  BCK(c->site_planes.ensure((size_t)n_site * kBoxPlanes), "alloc");
  BCK(c->site_nplanes.ensure((size_t)n_site), "alloc");
  BCK(c->centroid.ensure((size_t)n_tet), "alloc");
  BCK(c->tet_count.ensure((size_t)n_tet), "alloc");
  BCK(c->scratch.ensure(40), "alloc");
  // meshes to lanes, largest first onto the least loaded lane
  std::vector<int> order(b->meshes.size());
  for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
  auto work = [&](int i) { return (double)b->meshes[(size_t)i].n_tet + 4.0 * b->meshes[(size_t)i].n_site; };
  std::sort(order.begin(), order.end(), [&](int x, int y) { return work(x) > work(y); });
  double load[kFrontLanes] = {0};
  for (FrontLane& L : b->lanes) L.meshes.clear();
  for (int i : order) {
    int best = 0;
    for (int l = 1; l < kFrontLanes; ++l)
      if (load[l] < load[best]) best = l;
    load[best] += work(i);
    b->lanes[best].meshes.push_back(i);
  }
  for (FrontLane& L : b->lanes) {
    if (!L.stream) BCK(cudaStreamCreateWithFlags(&L.stream, cudaStreamNonBlocking), "stream");
    if (!L.done) BCK(cudaEventCreateWithFlags(&L.done, cudaEventDisableTiming), "event");
    long long max_sc = 1, max_tc = 1, max_site = 1, max_tet = 1;
    for (int i : L.meshes) {
      BatchMesh& m = b->meshes[(size_t)i];
      m.site_grid = rpd_make_grid(m.site_lo, m.site_hi, m.n_site, 2.0);
      max_sc = std::max<long long>(max_sc, (long long)m.site_grid.nx * m.site_grid.ny * m.site_grid.nz);
      for (int cl = 0; cl < 2; ++cl) {
        if (m.class_count[cl] == 0) continue;
        m.tet_grid[cl] = rpd_make_grid(m.mesh_lo, m.mesh_hi, m.class_count[cl], kTetsPerCell);
        const Grid& g = m.tet_grid[cl];
        max_tc = std::max<long long>(max_tc, (long long)g.nx * g.ny * g.nz);
      }
      max_site = std::max<long long>(max_site, m.n_site);
      max_tet = std::max<long long>(max_tet, m.n_tet);
    }
    BCK(L.s_cell_count.ensure((size_t)max_sc), "alloc");
    BCK(L.s_cell_start.ensure((size_t)max_sc + 1), "alloc");
    BCK(L.s_cell_fill.ensure((size_t)max_sc), "alloc");
    BCK(L.s_cell_items.ensure((size_t)max_site), "alloc");
    BCK(L.t_cell_of.ensure((size_t)max_tet), "alloc");
    BCK(L.t_cell_items.ensure((size_t)max_tet), "alloc");
    BCK(L.t_cell_count.ensure((size_t)max_tc), "alloc");
    BCK(L.t_cell_rmax.ensure((size_t)max_tc), "alloc");
    BCK(L.t_cell_start.ensure((size_t)max_tc + 1), "alloc");
    BCK(L.t_cell_fill.ensure((size_t)max_tc), "alloc");
    const long long scan_n = std::max(std::max(max_sc, max_tc), std::max(max_site, max_tet)) + 1;
    BCK(L.scan_tmp.ensure(scan_temp_ints(scan_n) + 16), "alloc");
    BCK(L.pair_ntasks.ensure((size_t)max_site), "alloc");
    BCK(L.pair_taskoff.ensure((size_t)max_site + 1), "alloc");
    BCK(L.work.ensure(1), "alloc");
  }
  if (!b->fork) BCK(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming), "event");
  std::vector<int32_t> tb(b->meshes.size());
  for (size_t m = 0; m < b->meshes.size(); ++m) tb[m] = b->meshes[m].tet_base;
  BCK(b->tet_base_dev.ensure(tb.size()), "alloc");
  BCK(cudaMemcpy(b->tet_base_dev.ptr, tb.data(), tb.size() * 4, cudaMemcpyHostToDevice), "H2D");
  BCK(b->mesh_first_dev.ensure(b->meshes.size() + 1), "alloc");
  // tet centroids (and radii) do not change: once
  BCK(c->tet_xyz.ensure((size_t)n_tet * 3), "alloc");
  BCK(c->tet_vadj.ensure((size_t)n_tet), "alloc");
  BCK(tet_centroids(c->vert3f.ptr, c->tets.ptr, n_tet, c->centroid.ptr, st, c->tet_xyz.ptr,
                    c->v_adjs.ptr, c->tet_vadj.ptr),
      "centroids");
  long long cap = c->pair_cap_hint > 0 ? c->pair_cap_hint : std::max<long long>(1 << 20, 8ll * n_tet);
  BCK(c->pair_buf.ensure((size_t)cap), "alloc pairs");
  BCK(cudaStreamSynchronize(st), "upload sync");
  drop_graph(b);
  b->uploaded = true;
  return RPD_OK;
}

// the front end of every mesh, enqueued on the context's stream (captured
// into a graph): neighbour lists, candidate boxes, candidate pairs
rpd_status front_end(rpd_batch* b) {
  rpd_ctx* c = b->ctx;
  cudaStream_t st = c->stream;
  const int k = c->k;
  BCK(cudaMemsetAsync(c->scratch.ptr, 0, 32 * sizeof(unsigned long long), st), "memset");
  BCK(cudaMemsetAsync(c->tet_count.ptr, 0, sizeof(int32_t) * (size_t)c->n_tet, st), "memset");
  const double u = std::ldexp(1.0, -24);
  BCK(cudaEventRecord(b->fork, st), "fork");
  for (FrontLane& L : b->lanes) {
   if (L.meshes.empty()) continue;
   BCK(cudaStreamWaitEvent(L.stream, b->fork, 0), "fork wait");
   const cudaStream_t ls = L.stream;
   for (int mi : L.meshes) {
    const BatchMesh& m = b->meshes[(size_t)mi];
    const int sb = m.site_base, tb = m.tet_base;
    // neighbour lists: the mesh's own site grid, ids offset to the batch
    BCK(grid_build_sites(c->site4f.ptr + sb, m.n_site, m.site_grid, c->s_cell_of.ptr + sb,
                         L.s_cell_count.ptr, L.s_cell_start.ptr, L.s_cell_fill.ptr,
                         L.s_cell_items.ptr, L.scan_tmp.ptr, ls), "site grid");
    BCK(launch_knn(c->site4f.ptr + sb, m.n_site, m.site_grid, L.s_cell_start.ptr,
                   L.s_cell_items.ptr, k, m.w_max, c->cfg.clip_order == RPD_ORDER_SITE_ID ? 1 : 0,
                   c->nbr.ptr + (long long)sb * k, c->nbr_keys.ptr + (long long)sb * k,
                   c->nbr_dist.ptr + (long long)sb * k, c->knn_status.ptr + sb, ls, sb,
                   c->nbr_bound.ptr + sb),
        "knn");
    // candidate pairs per radius class (as rpd_compute, with this mesh's bounds)
    double diag2 = 0.0, cs = 0.0, ext = 0.0;
    for (int a = 0; a < 3; ++a) {
      const double l = std::min(m.mesh_lo[a], m.site_lo[a]), h = std::max(m.mesh_hi[a], m.site_hi[a]);
      diag2 += (h - l) * (h - l);
      cs = std::max(cs, std::max(std::fabs(l), std::fabs(h)));
      ext = std::max(ext, m.mesh_hi[a] - m.mesh_lo[a]);
    }
    const double margin = 1e-4 * ext + 1e-6 * cs;
    const int box0 = c->cfg.box_planes > 0 ? c->cfg.box_planes : kDefaultBoxPlanes;
    for (int cl = 0; cl < 2; ++cl) {
      if (m.class_count[cl] == 0) continue;
      const Grid& tg = m.tet_grid[cl];
      BCK(grid_build_tets(c->centroid.ptr + tb, m.n_tet, c->tet_class.ptr + tb, cl, tg,
                          L.t_cell_of.ptr, L.t_cell_count.ptr, L.t_cell_start.ptr,
                          L.t_cell_fill.ptr, L.t_cell_items.ptr, L.scan_tmp.ptr, ls,
                          L.t_cell_rmax.ptr),
          "tet grid");
      const double R = m.class_radius[cl] * (1.0 + 1e-5) + 1e-6 * cs;
      BoxParams bp;
      bp.site4f = c->site4f.ptr;
      bp.flags = c->flags.ptr;
      bp.site_base = sb;
      bp.nbr = c->nbr_dist.ptr + (long long)sb * k;
      bp.k = k;
      bp.k_box = std::min(k, cl == 0 ? box0 : std::min(box0, 12));
      bp.n_site = m.n_site;
      bp.box_lo = make_float4((float)(m.mesh_lo[0] - margin), (float)(m.mesh_lo[1] - margin),
                              (float)(m.mesh_lo[2] - margin), 0.f);
      bp.box_hi = make_float4((float)(m.mesh_hi[0] + margin), (float)(m.mesh_hi[1] + margin),
                              (float)(m.mesh_hi[2] + margin), 0.f);
      bp.offset_r = (float)R;
      bp.offset_e = (float)(48.0 * u * (diag2 + std::fabs((double)m.w_max)));
      bp.coord_scale = (float)cs;
      bp.abs_margin = (float)margin;
      bp.site_box = c->site_box.ptr + 2ll * sb;
      bp.site_planes = c->site_planes.ptr + (long long)sb * kBoxPlanes;
      bp.site_nplanes = c->site_nplanes.ptr + sb;
      bp.counters = nullptr;
      const int bw = 4;
      const int bblocks = std::max(1, std::min((m.n_site + bw - 1) / bw, c->num_sms * box_blocks_per_sm(bw)));
      BCK(launch_site_box(bp, bblocks, bw, ls), "site boxes");
      PairParams pp;
      pp.vert3f = c->vert3f.ptr;
      pp.tets = c->tets.ptr + tb;
      pp.centroid = c->centroid.ptr + tb;
      pp.tet_xyz = c->tet_xyz.ptr + 3ll * tb;
      pp.tet_base = tb;
      pp.site_base = sb;
      pp.tg = tg;
      pp.tcell_start = L.t_cell_start.ptr;
      pp.tcell_items = L.t_cell_items.ptr;
      pp.tcell_rmax = L.t_cell_rmax.ptr;
      pp.site4f = c->site4f.ptr;
      pp.flags = c->flags.ptr;
      pp.nbr = c->nbr.ptr + (long long)sb * k;
      pp.rule_nbr = c->nbr_dist.ptr + (long long)sb * k;
      pp.k = k;
      pp.n_site = m.n_site;
      pp.site_box = c->site_box.ptr + 2ll * sb;
      pp.offset_r = bp.offset_r;
      pp.rule_keys = nullptr;  // (the rule checks every neighbour)
      pp.site_planes = c->site_planes.ptr + (long long)sb * kBoxPlanes;
      pp.site_nplanes = c->site_nplanes.ptr + sb;
      pp.coord_scale = (float)cs;
      pp.pair_buf = c->pair_buf.ptr;
      pp.pair_cursor = c->scratch.ptr + 4;
      pp.pair_cap = (long long)c->pair_buf.cap;
      pp.tet_count = c->tet_count.ptr;
      pp.diag = c->scratch.ptr + 20;
      BCK(launch_pairs(pp, L.pair_ntasks.ptr, L.pair_taskoff.ptr, L.scan_tmp.ptr, L.work.ptr,
                       c->num_sms, ls), "pairs");
    }
   }
   BCK(cudaEventRecord(L.done, ls), "join");
   BCK(cudaStreamWaitEvent(st, L.done, 0), "join wait");
  }
  return RPD_OK;
}

}  // namespace

extern "C" {

rpd_status rpd_batch_create(const rpd_config* cfg, rpd_batch** out) {
  if (!out) return RPD_ERR_INVALID_ARGUMENT;
  *out = nullptr;
  rpd_config c0;
  rpd_config_default(&c0);
  if (cfg) c0 = *cfg;
  if (c0.neighbor_source != RPD_NEIGH_KNN || c0.learned_k) return RPD_ERR_INVALID_ARGUMENT;
  rpd_ctx* c = nullptr;
  rpd_status s = rpd_create(&c0, &c);
  if (s != RPD_OK) return s;
  rpd_batch* b = new rpd_batch();
  b->ctx = c;
  *out = b;
  return RPD_OK;
}

void rpd_batch_destroy(rpd_batch* b) {
  if (!b) return;
  if (b->ctx) cudaSetDevice(b->ctx->device);
  drop_graph(b);
  for (FrontLane& L : b->lanes) {
    if (L.stream) {
      cudaStreamSynchronize(L.stream);
      cudaStreamDestroy(L.stream);
    }
    if (L.done) cudaEventDestroy(L.done);
  }
  if (b->fork) cudaEventDestroy(b->fork);
  rpd_destroy(b->ctx);
  delete b;
}

const char* rpd_batch_last_error(const rpd_batch* b) {
  if (!b) return "no batch";
  return b->err.empty() ? rpd_last_error(b->ctx) : b->err.c_str();
}

struct rpd_ctx* rpd_batch_context(rpd_batch* b) { return b ? b->ctx : nullptr; }

int rpd_batch_size(const rpd_batch* b) { return b ? (int)b->meshes.size() : 0; }

rpd_status rpd_batch_add_mesh(rpd_batch* b, const double* xyz, int n_vert, const int32_t* tets,
                              int n_tet, const int32_t* v_adjs, const uint8_t* e_adj6,
                              const int32_t* f_adjs, const int32_t* f_ids, const double* xyzw,
                              int n_site, const uint32_t* flags, int* mesh_index) {
  if (!b) return RPD_ERR_INVALID_ARGUMENT;
  b->err.clear();
  if (n_vert <= 0 || n_tet <= 0 || n_site <= 0 || !xyz || !tets || !v_adjs || !e_adj6 || !f_adjs ||
      !f_ids || !xyzw)
    return bfail(b, RPD_ERR_INVALID_ARGUMENT, "rpd_batch_add_mesh: empty mesh, no sites or null buffer");
  const long long tot_tet = (long long)b->tets.size() / 4 + n_tet;
  const long long tot_vert = (long long)b->xyz.size() / 3 + n_vert;
  const long long tot_site = (long long)b->sites.size() / 4 + n_site;
  if (tot_tet > INT32_MAX / 2 || tot_vert > INT32_MAX / 2 || tot_site > INT32_MAX / 2)
    return bfail(b, RPD_ERR_CAPACITY, "rpd_batch_add_mesh: batch too large");
  BatchMesh m;
  m.vert_base = (int)(b->xyz.size() / 3);
  m.tet_base = (int)(b->tets.size() / 4);
  m.site_base = (int)(b->sites.size() / 4);
  m.n_vert = n_vert;
  m.n_tet = n_tet;
  m.n_site = n_site;
  for (int a = 0; a < 3; ++a) {
    m.mesh_lo[a] = m.site_lo[a] = INFINITY;
    m.mesh_hi[a] = m.site_hi[a] = -INFINITY;
  }
  for (long long i = 0; i < (long long)n_vert * 3; ++i) {
    if (!std::isfinite(xyz[i])) return bfail(b, RPD_ERR_INVALID_ARGUMENT, "rpd_batch_add_mesh: non-finite vertex");
    m.mesh_lo[i % 3] = std::min(m.mesh_lo[i % 3], xyz[i]);
    m.mesh_hi[i % 3] = std::max(m.mesh_hi[i % 3], xyz[i]);
  }
  float wmax = -INFINITY;
  for (long long i = 0; i < n_site; ++i) {
    for (int a = 0; a < 4; ++a)
      if (!std::isfinite(xyzw[4 * i + a]))
        return bfail(b, RPD_ERR_INVALID_ARGUMENT, "rpd_batch_add_mesh: non-finite site");
    for (int a = 0; a < 3; ++a) {
      m.site_lo[a] = std::min(m.site_lo[a], xyzw[4 * i + a]);
      m.site_hi[a] = std::max(m.site_hi[a], xyzw[4 * i + a]);
    }
    wmax = std::max(wmax, (float)xyzw[4 * i + 3]);
  }
  m.w_max = wmax;
  // tet radii and this mesh's two radius classes (99.5th percentile split)
  std::vector<double> rad((size_t)n_tet);
  for (long long t = 0; t < n_tet; ++t) {
    double cen[3] = {0, 0, 0};
    for (int q = 0; q < 4; ++q) {
      const int v = tets[4 * t + q];
      if (v < 0 || v >= n_vert)
        return bfail(b, RPD_ERR_INVALID_ARGUMENT, "rpd_batch_add_mesh: vertex id out of range");
      for (int a = 0; a < 3; ++a) cen[a] += 0.25 * xyz[3 * (long long)v + a];
    }
    double r = 0.0;
    for (int q = 0; q < 4; ++q) {
      const int v = tets[4 * t + q];
      double d2 = 0.0;
      for (int a = 0; a < 3; ++a) {
        const double d = xyz[3 * (long long)v + a] - cen[a];
        d2 += d * d;
      }
      r = std::max(r, std::sqrt(d2));
    }
    rad[(size_t)t] = r;
  }
  std::vector<double> tmp(rad);
  const size_t qi = std::min(tmp.size() - 1, (size_t)(0.995 * (double)tmp.size()));
  std::nth_element(tmp.begin(), tmp.begin() + qi, tmp.end());
  const double r0 = tmp[qi];
  for (long long t = 0; t < n_tet; ++t) {
    const int cl = rad[(size_t)t] <= r0 ? 0 : 1;
    b->tet_class.push_back((uint8_t)cl);
    m.class_count[cl]++;
    m.class_radius[cl] = std::max(m.class_radius[cl], rad[(size_t)t]);
  }
  b->xyz.insert(b->xyz.end(), xyz, xyz + 3ll * n_vert);
  for (long long i = 0; i < 4ll * n_tet; ++i) b->tets.push_back(tets[i] + m.vert_base);
  b->v_adjs.insert(b->v_adjs.end(), v_adjs, v_adjs + n_vert);
  b->e_adj6.insert(b->e_adj6.end(), e_adj6, e_adj6 + 6ll * n_tet);
  b->f_adjs.insert(b->f_adjs.end(), f_adjs, f_adjs + 4ll * n_tet);
  b->f_ids.insert(b->f_ids.end(), f_ids, f_ids + 4ll * n_tet);
  b->sites.insert(b->sites.end(), xyzw, xyzw + 4ll * n_site);
  for (long long i = 0; i < n_site; ++i) b->flags.push_back(flags ? flags[i] : 1u);
  if (mesh_index) *mesh_index = (int)b->meshes.size();
  b->meshes.push_back(m);
  b->uploaded = false;
  return RPD_OK;
}

rpd_status rpd_batch_set_graph(rpd_batch* b, int use_graph) {
  if (!b || (use_graph != 0 && use_graph != 1)) return RPD_ERR_INVALID_ARGUMENT;
  b->use_graph = use_graph != 0;
  if (!b->use_graph) drop_graph(b);
  return RPD_OK;
}

rpd_status rpd_batch_compute(rpd_batch* b, rpd_stats* stats) {
  if (!b) return RPD_ERR_INVALID_ARGUMENT;
  b->err.clear();
  if (b->meshes.empty()) return bfail(b, RPD_ERR_NOT_READY, "rpd_batch_compute: no meshes");
  rpd_ctx* c = b->ctx;
  if (c->cfg.neighbor_source != RPD_NEIGH_KNN || c->cfg.learned_k)
    return bfail(b, RPD_ERR_INVALID_ARGUMENT, "rpd_batch_compute: GPU-built lists, no learned_k");
  BCK(cudaSetDevice(c->device), "cudaSetDevice");
  if (!b->uploaded) {
    rpd_status s = upload(b);
    if (s != RPD_OK) return s;
  }
  cudaStream_t st = c->stream;
  if (c->cfg.knn_k != c->k) {  // list length changed: buffers resized
    rpd_status s = upload(b);
    if (s != RPD_OK) return s;
  }
  if (b->exec && (b->captured_cfg.knn_k != c->cfg.knn_k ||
                  b->captured_cfg.clip_order != c->cfg.clip_order ||
                  b->captured_cfg.box_planes != c->cfg.box_planes))
    drop_graph(b);
  for (int attempt = 0; attempt < 3; ++attempt) {
    take_launches();
    BCK(cudaEventRecord(c->ev[kEvStart], st), "event");
    if (b->use_graph) {
      if (!b->exec) {
        BCK(cudaStreamBeginCapture(st, cudaStreamCaptureModeRelaxed), "capture");
        rpd_status s = front_end(b);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(st, &g);
        if (s != RPD_OK) {
          if (g) cudaGraphDestroy(g);
          return s;
        }
        BCK(e, "end capture");
        b->graph = g;
        BCK(cudaGraphInstantiate(&b->exec, g, 0), "graph instantiate");
        b->captured_cfg = c->cfg;
        b->graph_launches = take_launches();
      }
      BCK(cudaGraphLaunch(b->exec, st), "graph launch");
      note_launches(b->graph_launches);
    } else {
      rpd_status s = front_end(b);
      if (s != RPD_OK) return s;
    }
    BCK(cudaEventRecord(c->ev[kEvKnn], st), "event");
    unsigned long long np = 0;
    BCK(cudaMemcpyAsync(&np, c->scratch.ptr + 4, sizeof(np), cudaMemcpyDeviceToHost, st), "D2H");
    BCK(cudaStreamSynchronize(st), "front end sync");
    c->n_pairs = (long long)np;
    if ((long long)np <= (long long)c->pair_buf.cap) break;
    // more pairs than the buffer holds: grow it and record the front end again
    drop_graph(b);
    BCK(c->pair_buf.ensure((size_t)(np + np / 8 + 1024)), "alloc pairs");
    if (attempt == 2) return bfail(b, RPD_ERR_CAPACITY, "rpd_batch_compute: pair buffer");
  }
  if (c->n_pairs > INT32_MAX) return bfail(b, RPD_ERR_CAPACITY, "rpd_batch_compute: more than 2^31 pairs");
  c->pair_cap_hint = std::max<long long>(c->pair_cap_hint, c->n_pairs + c->n_pairs / 8 + 1024);
  // exact lists: the rounds search one grid of every site of the batch, each
  // site restricted to its mesh's ids
  const bool exact = c->cfg.exact_lists != 0;
  if (exact) {
    const int n_site = c->n_site;
    const Grid g = rpd_make_grid(c->grid_lo, c->grid_hi, n_site, 2.0);
    const long long nc = (long long)g.nx * g.ny * g.nz;
    BCK(c->s_cell_count.ensure((size_t)nc), "alloc");
    BCK(c->s_cell_start.ensure((size_t)nc + 1), "alloc");
    BCK(c->s_cell_fill.ensure((size_t)nc), "alloc");
    BCK(c->s_cell_items.ensure((size_t)n_site), "alloc");
    BCK(c->scan_tmp.ensure(scan_temp_ints(std::max<long long>(nc, n_site)) + 16), "alloc");
    BCK(grid_build_sites(c->site_gridpos.ptr, n_site, g, c->s_cell_of.ptr, c->s_cell_count.ptr,
                         c->s_cell_start.ptr, c->s_cell_fill.ptr, c->s_cell_items.ptr,
                         c->scan_tmp.ptr, st), "site grid");
  }
  rpd_status s = rpd_finish_compute(c, true, false, stats, exact);
  c->cells_for_mesh = false;  // a batch's cells are not one mesh's (no partial update)
  if (s != RPD_OK) return bfail(b, s, rpd_last_error(c));
  // first compacted cell of every mesh
  const int nm = (int)b->meshes.size();
  BCK(mesh_cell_ranges(c->cells.ptr, c->n_out.ptr, b->tet_base_dev.ptr, nm, b->mesh_first_dev.ptr, st),
      "ranges");
  b->mesh_first.assign((size_t)nm + 1, 0);
  BCK(cudaMemcpyAsync(b->mesh_first.data(), b->mesh_first_dev.ptr, sizeof(long long) * (nm + 1),
                      cudaMemcpyDeviceToHost, st), "D2H");
  BCK(cudaStreamSynchronize(st), "ranges sync");
  return RPD_OK;
}

rpd_status rpd_batch_mesh_cells(rpd_batch* b, int mesh, int64_t* first_cell, int64_t* n_cells) {
  if (!b || mesh < 0 || mesh >= (int)b->meshes.size()) return RPD_ERR_INVALID_ARGUMENT;
  if (!b->ctx->has_result || b->mesh_first.size() != b->meshes.size() + 1)
    return bfail(b, RPD_ERR_NOT_READY, "rpd_batch_mesh_cells: no result");
  if (first_cell) *first_cell = b->mesh_first[(size_t)mesh];
  if (n_cells) *n_cells = b->mesh_first[(size_t)mesh + 1] - b->mesh_first[(size_t)mesh];
  return RPD_OK;
}

rpd_status rpd_batch_copy_mesh_cells(rpd_batch* b, int mesh, rpd_cell_header* headers,
                                     int64_t max_cells, void* payload, int64_t payload_capacity,
                                     int64_t* n_cells_out, int64_t* payload_bytes_out) {
  int64_t first = 0, n = 0;
  rpd_status s = rpd_batch_mesh_cells(b, mesh, &first, &n);
  if (s != RPD_OK) return s;
  rpd_ctx* c = b->ctx;
  BCK(cudaSetDevice(c->device), "cudaSetDevice");
  cudaStream_t st = c->stream;
  std::vector<rpd_cell_header> h((size_t)std::max<int64_t>(n, 1));
  if (n > 0)
    BCK(cudaMemcpy(h.data(), c->cells.ptr + first, sizeof(rpd_cell_header) * (size_t)n,
                   cudaMemcpyDeviceToHost), "D2H");
  std::vector<unsigned long long> off((size_t)std::max<int64_t>(n, 1));
  unsigned long long bytes = 0;
  for (int64_t q = 0; q < n; ++q) {
    off[(size_t)q] = bytes;
    bytes += PayloadLayout(h[(size_t)q].nb_v, h[(size_t)q].nb_p, h[(size_t)q].nb_e).total;
  }
  if (n_cells_out) *n_cells_out = n;
  if (payload_bytes_out) *payload_bytes_out = (int64_t)bytes;
  if (!headers && !payload) return RPD_OK;
  if (!headers || !payload || max_cells < n || payload_capacity < (int64_t)bytes)
    return bfail(b, RPD_ERR_CAPACITY, "rpd_batch_copy_mesh_cells: buffers too small");
  if (n == 0) return RPD_OK;
  DevBuf<unsigned long long> doff;
  DevBuf<rpd_cell_header> dh;
  DevBuf<uint8_t> dp;
  BCK(doff.ensure((size_t)n), "alloc");
  BCK(dh.ensure((size_t)n), "alloc");
  BCK(dp.ensure((size_t)bytes), "alloc");
  BCK(cudaMemcpyAsync(doff.ptr, off.data(), sizeof(unsigned long long) * (size_t)n,
                      cudaMemcpyHostToDevice, st), "H2D");
  const BatchMesh& m = b->meshes[(size_t)mesh];
  BCK(gather_records(c->cells.ptr + first, n, doff.ptr, c->payload.ptr, m.tet_base, m.site_base,
                     dh.ptr, dp.ptr, st), "gather");
  BCK(cudaMemcpyAsync(headers, dh.ptr, sizeof(rpd_cell_header) * (size_t)n, cudaMemcpyDeviceToHost, st), "D2H");
  BCK(cudaMemcpyAsync(payload, dp.ptr, (size_t)bytes, cudaMemcpyDeviceToHost, st), "D2H");
  BCK(cudaStreamSynchronize(st), "copy sync");
  return RPD_OK;
}

rpd_status rpd_batch_autotune(rpd_batch* b, int repeats, rpd_tuning* result) {
  if (!b) return RPD_ERR_INVALID_ARGUMENT;
  if (repeats < 1) repeats = 1;
  rpd_ctx* c = b->ctx;
  if (b->meshes.empty()) return bfail(b, RPD_ERR_NOT_READY, "rpd_batch_autotune: no meshes");
  if (!b->uploaded) {
    rpd_status s = upload(b);
    if (s != RPD_OK) return s;
  }
  struct Cand {
    int warps, variant, bucket;
  };
  const rpd_config saved = c->cfg;
  std::vector<Cand> cands = {{saved.warps_per_block > 0 ? saved.warps_per_block : 4, saved.clip_variant, 0},
                             {2, 0, 0}, {4, 0, 0}, {8, 0, 0}, {4, 1, 0}, {4, 2, 0}};
  std::vector<int> buckets = {0};
  if (c->cfg.certify) {
    buckets.push_back(16);
    buckets.push_back(32);
  }
  float best = INFINITY, first = 0.f;
  Cand best_c = cands[0];
  int tried = 0;
  for (int bk : buckets) {
    for (size_t ci = 0; ci < cands.size(); ++ci) {
      if (bk != 0 && ci == 0) continue;
      Cand cd = cands[ci];
      cd.bucket = bk;
      c->cfg.warps_per_block = cd.warps;
      c->cfg.clip_variant = cd.variant;
      c->cfg.blocks_per_sm = 0;
      if (bk > 0) {
        std::vector<int32_t> kk((size_t)c->n_site, bk);
        rpd_status s = rpd_set_site_k(c, kk.data(), 0);
        if (s != RPD_OK) return bfail(b, s, rpd_last_error(c));
      } else {
        c->has_site_klen = false;
      }
      std::vector<float> t;
      for (int r = 0; r < repeats + 1; ++r) {
        rpd_stats st;
        rpd_status s = rpd_batch_compute(b, &st);
        if (s != RPD_OK) {
          c->cfg = saved;
          return s;
        }
        if (r > 0) t.push_back(st.ms_clip);
      }
      std::sort(t.begin(), t.end());
      const float med = t[t.size() / 2];
      if (tried == 0) first = med;
      ++tried;
      if (med < best) {
        best = med;
        best_c = cd;
      }
    }
  }
  c->cfg = saved;
  c->cfg.warps_per_block = best_c.warps;
  c->cfg.clip_variant = best_c.variant;
  c->cfg.blocks_per_sm = 0;
  if (best_c.bucket > 0) {
    std::vector<int32_t> kk((size_t)c->n_site, best_c.bucket);
    rpd_status s = rpd_set_site_k(c, kk.data(), 0);
    if (s != RPD_OK) return bfail(b, s, rpd_last_error(c));
  } else {
    c->has_site_klen = false;
  }
  c->has_result = false;
  if (result) {
    result->warps_per_block = best_c.warps;
    result->clip_variant = best_c.variant;
    result->k_bucket = best_c.bucket;
    result->n_candidates = tried;
    result->ms_clip_best = best;
    result->ms_clip_first = first;
    result->learned_k = 0;
  }
  return RPD_OK;
}

}  // extern "C"
