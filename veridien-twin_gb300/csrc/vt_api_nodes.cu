// C ABI of the scene's node radiosity (include/vtwin.h, "scene node radiosity"): the gather-table build and the
// update bookkeeping of gpu/renderer.js:456-531 (_buildGatherTable), :713-822 (_submitNodeDirect, _submitJacobi,
// _movedSinceSolve, _ensureRadiosity, converge) and :825-851 (nodeSummary), around the kernels of vt_nodes.cu.
#include <chrono>

#include "vt_ctx.cuh"
#include "vt_nodes.cuh"

using namespace vtapi;

namespace {

vt_nodes_opts default_opts() {
  vt_nodes_opts o{};
  o.gather_k = 64; o.node_samples = 4; o.nbr_k = 16; o.smooth_sigma = 0.003f; o.smooth_radius = 0.006f;
  o.radiosity_every = 1; o.iters_per_frame = 4; o.iters_initial = 96;
  return o;
}

size_t al(size_t b) { return (b + 255) & ~size_t(255); }

// bodies whose pose differs from the last update; all = the emitter body moved (or nothing was solved yet)
void moved_since_solve(const vt_ctx* ctx, bool& all, uint32_t& mask) {
  const auto& N = ctx->nodes;
  all = false;
  mask = 0;
  if (N.solved_inst.size() != ctx->inst.size()) { all = true; return; }
  for (size_t i = 0; i < ctx->inst.size(); i++) {
    const vt::InstPose &I = ctx->inst[i], &L = N.solved_inst[i];
    bool same = !I.valid && !L.valid;
    if (I.valid && L.valid) {
      same = true;
      for (int k = 0; k < 4; k++) same = same && std::fabs(I.q0[k] - L.q0[k]) < 1e-9 && std::fabs(I.q1[k] - L.q1[k]) < 1e-9;
      for (int k = 0; k < 3; k++) same = same && std::fabs(I.p0[k] - L.p0[k]) < 1e-10 && std::fabs(I.p1[k] - L.p1[k]) < 1e-10;
    }
    if (!same) {
      mask |= 1u << i;
      if (int(i) == ctx->S.scope_index) all = true;
    }
  }
}

// the poses and bounding capsules of this update, for the next incremental one
void snapshot(vt_ctx* ctx) {
  auto& N = ctx->nodes;
  N.solved_inst = ctx->inst;
  const size_t nb = ctx->S.bodies.size();
  N.solved_caps.assign(nb * 8, 0.0f);
  for (size_t i = 0; i < nb; i++)
    for (int k = 0; k < 8; k++) N.solved_caps[8 * i + k] = ctx->su_host[vt::SU_INST + 48 * i + 32 + k];
}

}  // namespace

vt_status vt_nodes_build(vt_ctx* ctx, const vt_nodes_opts* opts, vt_nodes_info* info) {
  if (!ctx) return VT_ERR_ARG;
  vt_nodes_opts o = opts ? *opts : default_opts();
  if (o.gather_k < 1 || o.gather_k > 1024 || o.nbr_k < 1 || o.nbr_k > 64 || o.node_samples < 1 || o.node_samples > 4096)
    return fail(ctx, VT_ERR_ARG, "nodes: gather_k 1..1024, nbr_k 1..64, node_samples 1..4096");
  if (!(o.smooth_radius > 0.0f) || !(o.smooth_sigma >= 0.0f)) return fail(ctx, VT_ERR_ARG, "nodes: smooth_radius > 0, smooth_sigma >= 0");
  if (o.radiosity_every < 1) o.radiosity_every = 1;
  auto& N = ctx->nodes;
  const uint32_t n = ctx->S.static_verts, K = o.gather_k;
  const uint32_t n_mat = uint32_t(std::max<size_t>(1, ctx->S.mats.size()));
  const size_t b_g = al(size_t(n) * K * 4), b_aux = al(size_t(n) * 16 + 16), b_act = al(size_t(n) * 4 + 4),
               b_nbr = al(size_t(n) * o.nbr_k * 8 + 8), b_amu = al(size_t(n_mat) * K * 16);
  VT_CK(cudaStreamSynchronize(ctx->stream));
  cudaFree(N.mem);
  cudaFree(N.table_mem);
  cudaFree(N.direct_mem);
  N = vt_ctx::Nodes{};
  if (cudaMalloc(&N.mem, b_g + b_aux + b_act + b_nbr + b_amu) != cudaSuccess) {
    cudaGetLastError();
    N.mem = nullptr;
    return fail(ctx, VT_ERR_OOM, "nodes: gather table allocation failed");
  }
  char* p = static_cast<char*>(N.mem);
  N.gtable = reinterpret_cast<uint32_t*>(p); p += b_g;
  N.aux = reinterpret_cast<float4*>(p); p += b_aux;
  N.active = reinterpret_cast<uint32_t*>(p); p += b_act;
  N.nbr = reinterpret_cast<uint2*>(p); p += b_nbr;
  N.amu = reinterpret_cast<float4*>(p);
  N.o = o;
  N.n = n;
  N.n_mat = n_mat;
  // the node state starts over: V = 1, visibility code -1 (gpu/renderer.js:322-327)
  std::vector<float> st(std::max<size_t>(16, size_t(n) * 16), 0.0f);
  for (uint32_t i = 0; i < n; i++) { st[16 * size_t(i) + 3] = 1; st[16 * size_t(i) + 15] = -1; }
  VT_CK(cudaMemcpyAsync(ctx->d_nstate, st.data(), size_t(n) * 64, cudaMemcpyHostToDevice, ctx->stream));
  ctx->slot = 1;
  vt_status s = write_su(ctx);
  if (s != VT_OK) return s;
  const vtd::Scene S = dev_scene(ctx);
  VT_CK(cudaEventRecord(ctx->ev0, ctx->stream));
  if (n) vtk::launch_gather_build(S, n, K, N.gtable, N.aux, ctx->stream);
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->ev1, ctx->stream));
  std::vector<float4> aux(n);
  if (n) VT_CK(cudaMemcpyAsync(aux.data(), N.aux, size_t(n) * 16, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  float ms = 0;
  cudaEventElapsedTime(&ms, ctx->ev0, ctx->ev1);
  N.build_ms = ms;
  // active nodes: at most half their gather rays escape
  N.misses.resize(n);
  for (uint32_t i = 0; i < n; i++) {
    N.misses[i] = aux[i].x;
    if (aux[i].x <= 0.5f * float(K)) N.active_h.push_back(i);
  }
  N.n_active = uint32_t(N.active_h.size());
  if (cudaMalloc(&N.direct_mem, vtk::node_direct_bytes(N.n_active, o.node_samples)) != cudaSuccess) {
    cudaGetLastError();
    N.direct_mem = nullptr;
    return fail(ctx, VT_ERR_OOM, "nodes: direct-light buffers");
  }
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<uint32_t> nbr;
  vt::node_neighbours(ctx->S, N.active_h, o.nbr_k, double(o.smooth_radius), double(o.smooth_sigma), nbr);
  N.nbr_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  if (N.n_active) {
    VT_CK(cudaMemcpyAsync(N.active, N.active_h.data(), size_t(N.n_active) * 4, cudaMemcpyHostToDevice, ctx->stream));
    VT_CK(cudaMemcpyAsync(N.nbr, nbr.data(), nbr.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
  }
  vtk::launch_amu(S, n_mat, K, N.amu, ctx->stream);
  VT_CK(cudaGetLastError());
  // the transport table: row offsets from the landing-ray counts (aux holds the counts for a moment), then entries
  if (!o.per_step_factors && N.n_active) {
    uint32_t* cnt_d = reinterpret_cast<uint32_t*>(N.aux);
    vtk::launch_transport_count(N.active, N.n_active, K, N.gtable, cnt_d, ctx->stream);
    std::vector<uint32_t> cnt(N.n_active), row(size_t(N.n_active) + 1, 0u);
    VT_CK(cudaMemcpyAsync(cnt.data(), cnt_d, size_t(N.n_active) * 4, cudaMemcpyDeviceToHost, ctx->stream));
    VT_CK(cudaStreamSynchronize(ctx->stream));
    uint64_t nnz = 0;
    for (uint32_t k = 0; k < N.n_active; k++) { row[k] = uint32_t(nnz); nnz += cnt[k]; }
    const size_t b_row = al((size_t(N.n_active) + 1) * 4);
    if (nnz < (uint64_t(1) << 32) && cudaMalloc(&N.table_mem, b_row + size_t(nnz) * 16 + 16) == cudaSuccess) {
      row[N.n_active] = uint32_t(nnz);
      N.row = static_cast<uint32_t*>(N.table_mem);
      N.ent = reinterpret_cast<float4*>(static_cast<char*>(N.table_mem) + b_row);
      N.nnz = nnz;
      VT_CK(cudaMemcpyAsync(N.row, row.data(), row.size() * 4, cudaMemcpyHostToDevice, ctx->stream));
      vtk::launch_transport_fill(S, N.active, N.n_active, K, N.gtable, N.amu, N.row, N.ent, ctx->stream);
      VT_CK(cudaGetLastError());
    } else {
      cudaGetLastError();   // too large for the device: the factors are evaluated per step
      N.table_mem = nullptr;
    }
  }
  VT_CK(cudaStreamSynchronize(ctx->stream));
  N.built = true;
  N.auto_update = true;
  if (info) {
    info->n_nodes = n; info->n_active = N.n_active; info->gather_k = K; info->nbr_k = o.nbr_k;
    info->build_ms = N.build_ms; info->neighbour_ms = N.nbr_ms; info->table_entries = N.nnz;
  }
  return VT_OK;
}

vt_status vt_nodes_direct(vt_ctx* ctx, uint32_t moved) {
  if (!ctx) return VT_ERR_ARG;
  if (!ctx->nodes.built) return fail(ctx, VT_ERR_ARG, "nodes: vt_nodes_build first");
  VT_CK(cudaEventRecord(ctx->nev[0], ctx->stream));
  vtk::launch_node_direct(dev_scene(ctx), ctx->nodes.active, ctx->nodes.n_active, ctx->nodes.o.node_samples, moved, ctx->d_nstate,
                          ctx->nodes.direct_mem, ctx->wave_blocks, ctx->stream);
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->nev[1], ctx->stream));
  ctx->nodes.timed_direct = true;
  return VT_OK;
}

vt_status vt_nodes_jacobi(vt_ctx* ctx, uint32_t iters) {
  if (!ctx) return VT_ERR_ARG;
  auto& N = ctx->nodes;
  if (!N.built) return fail(ctx, VT_ERR_ARG, "nodes: vt_nodes_build first");
  const vtd::Scene S = dev_scene(ctx);
  uint32_t slot = ctx->slot ? ctx->slot : 1;
  VT_CK(cudaEventRecord(ctx->nev[2], ctx->stream));
  for (uint32_t k = 0; k < iters; k++) {
    const uint32_t out = slot == 1 ? 2 : 1;
    vtk::launch_jacobi_step(S, N.active, N.n_active, N.o.gather_k, N.gtable, N.amu, N.row, N.ent, N.nbr, N.o.nbr_k, slot, out,
                            ctx->d_nstate, N.aux, ctx->stream);
    slot = out;
  }
  VT_CK(cudaGetLastError());
  VT_CK(cudaEventRecord(ctx->nev[3], ctx->stream));
  N.timed_jacobi = true;
  N.last_steps = iters;
  ctx->slot = slot;
  return write_su(ctx);
}

vt_status vt_node_summary(vt_ctx* ctx, double out[13]) {
  if (!ctx) return VT_ERR_ARG;
  auto& N = ctx->nodes;
  if (!N.built) return fail(ctx, VT_ERR_ARG, "nodes: vt_nodes_build first");
  std::vector<float> st(size_t(N.n) * 16);
  if (N.n) VT_CK(cudaMemcpyAsync(st.data(), ctx->d_nstate, st.size() * 4, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  const uint32_t slot = ctx->slot ? ctx->slot : 1;
  double A = 0, E[3] = {0, 0, 0}, Ed[3] = {0, 0, 0}, Lo[3] = {0, 0, 0};
  for (uint32_t i : N.active_h) {
    const double a = ctx->S.node_area[i], V = st[16 * size_t(i) + 3];
    A += a;
    const uint32_t mesh = ctx->S.verts[8 * size_t(i) + 3];
    const double* hh = ctx->S.mats[ctx->S.meshes[mesh].mat].hh;
    for (int c = 0; c < 3; c++) {
      E[c] += a * st[16 * size_t(i) + c] * V;
      Lo[c] += a * st[16 * size_t(i) + 4 * slot + c] * std::max(1e-4, hh[c]);
      Ed[c] += a * st[16 * size_t(i) + 12 + c] / std::max(1e-3, hh[c]);
    }
  }
  double r[13] = {A};
  for (int c = 0; c < 3; c++) {
    const double inv = A > 0 ? 1.0 / A : 0.0;
    r[1 + c] = E[c] * inv; r[4 + c] = Ed[c] * inv; r[7 + c] = Lo[c] * inv; r[10 + c] = r[1 + c] + r[4 + c];
    ctx->eavg[c] = float(r[10 + c]);
  }
  if (out) std::memcpy(out, r, sizeof(r));
  return write_su(ctx);
}

vt_status vt_nodes_update(vt_ctx* ctx, int force, uint32_t* what) {
  if (!ctx) return VT_ERR_ARG;
  auto& N = ctx->nodes;
  if (what) *what = 0;
  if (!N.built || !N.n_active) return VT_OK;
  const int64_t pv = int64_t(N.poses_version);
  if (!force && N.solved_version == pv) return VT_OK;
  if (!force && N.solved_version >= 0 && pv - N.solved_version < int64_t(N.o.radiosity_every)) return VT_OK;
  const bool first = N.solved_version < 0;
  bool all = true;
  uint32_t mask = 0;
  if (!first && !force) moved_since_solve(ctx, all, mask);
  vt_status s;
  uint32_t w = 3;
  if (all || mask) {
    if ((s = vt_nodes_direct(ctx, all ? 0u : mask)) != VT_OK) return s;
    if ((s = vt_nodes_jacobi(ctx, first ? std::min<uint32_t>(N.o.iters_initial, 8) : N.o.iters_per_frame)) != VT_OK) return s;
    snapshot(ctx);
    w = all ? 1 : 2;
  }
  if (first) N.pending = int64_t(N.o.iters_initial) - 8;   // the rest of the first solve, 8 steps per later update
  else if (N.pending > 0) {
    if ((s = vt_nodes_jacobi(ctx, uint32_t(std::min<int64_t>(8, N.pending)))) != VT_OK) return s;
    N.pending -= 8;
  }
  N.solved_version = pv;
  if ((s = write_su(ctx)) != VT_OK) return s;
  // eAvg follows a full update, the first solve, and the end of the first solve
  if (all || first || (N.pending <= 0 && !N.eavg_settled)) {
    if (N.pending <= 0) N.eavg_settled = true;
    if ((s = vt_node_summary(ctx, nullptr)) != VT_OK) return s;
  }
  if (what) *what = w;
  return VT_OK;
}

vt_status vt_converge(vt_ctx* ctx, uint32_t iters) {
  if (!ctx) return VT_ERR_ARG;
  auto& N = ctx->nodes;
  if (!N.built) return fail(ctx, VT_ERR_ARG, "converge: vt_nodes_build first");
  vt_status s;
  if (N.solved_version != int64_t(N.poses_version)) {
    if ((s = vt_nodes_direct(ctx, 0)) != VT_OK) return s;
    N.solved_version = int64_t(N.poses_version);
    snapshot(ctx);
  }
  if ((s = vt_nodes_jacobi(ctx, iters)) != VT_OK) return s;
  N.pending = 0;
  N.auto_update = true;
  return vt_node_summary(ctx, nullptr);
}

vt_status vt_nodes_export(vt_ctx* ctx, uint32_t* gtable, uint32_t* active, uint32_t* nbr, float* misses) {
  if (!ctx) return VT_ERR_ARG;
  const auto& N = ctx->nodes;
  if (!N.built) return fail(ctx, VT_ERR_ARG, "nodes: vt_nodes_build first");
  if (gtable && N.n) VT_CK(cudaMemcpyAsync(gtable, N.gtable, size_t(N.n) * N.o.gather_k * 4, cudaMemcpyDeviceToHost, ctx->stream));
  if (nbr && N.n_active) VT_CK(cudaMemcpyAsync(nbr, N.nbr, size_t(N.n_active) * N.o.nbr_k * 8, cudaMemcpyDeviceToHost, ctx->stream));
  VT_CK(cudaStreamSynchronize(ctx->stream));
  if (active) std::copy(N.active_h.begin(), N.active_h.end(), active);
  if (misses) std::copy(N.misses.begin(), N.misses.end(), misses);
  return VT_OK;
}

vt_status vt_get_node_state(vt_ctx* ctx, float* state, uint32_t* slot) {
  if (!ctx) return VT_ERR_ARG;
  if (state && ctx->S.static_verts) {
    vt_status s = from_device(ctx, state, ctx->d_nstate, size_t(ctx->S.static_verts) * 64);
    if (s != VT_OK) return s;
    VT_CK(cudaStreamSynchronize(ctx->stream));
  }
  if (slot) *slot = ctx->slot;
  return VT_OK;
}
