// fsim_api.cu -- the C ABI (include/fsim.h): handle lifecycle, memory,
// particle I/O, per-stage entry points, the fused step and kernel timing.
#include <algorithm>
#include <cstdlib>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>

#include "fsim_internal.cuh"

namespace fsim {

int fail(fsim_sim* s, int code, const std::string& msg) {
  if (s) s->err = msg;
  return code;
}

int cuda_fail(fsim_sim* s, cudaError_t e, const char* what) {
  if (s) s->err = std::string(what) + ": " + cudaGetErrorString(e);
  return FSIM_ERR_CUDA;
}

ProfScope::ProfScope(fsim_sim* sim, const char* name) : s(sim) {
  if (!s->profiling) return;
  for (size_t i = 0; i < s->kstats.size(); ++i)
    if (std::strcmp(s->kstats[i].name, name) == 0) { idx = int(i); break; }
  if (idx < 0) {
    s->kstats.push_back(KernelStat{name, 0.0, 0});
    idx = int(s->kstats.size()) - 1;
  }
  auto take = [&]() {
    cudaEvent_t e = nullptr;
    if (!s->ev_pool.empty()) {
      e = s->ev_pool.back();
      s->ev_pool.pop_back();
    } else {
      cudaEventCreate(&e);
    }
    return e;
  };
  a = take();
  b = take();
  cudaEventRecord(a, s->stream);
}

ProfScope::~ProfScope() {
  if (idx < 0) return;
  cudaEventRecord(b, s->stream);
  s->pending.push_back(fsim_sim::Pending{idx, a, b});
}

namespace {

template <typename T>
int dmalloc(fsim_sim* s, T** p, size_t count) {
  *p = nullptr;
  if (count == 0) count = 1;
  cudaError_t e = cudaMalloc(reinterpret_cast<void**>(p), count * sizeof(T));
  if (e != cudaSuccess) return cuda_fail(s, e, "cudaMalloc");
  return FSIM_OK;
}

template <typename T>
void dfree(T*& p) {
  if (p) cudaFree(p);
  p = nullptr;
}

int resolve_profile(fsim_sim* s) {
  if (s->pending.empty()) return FSIM_OK;
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  for (auto& p : s->pending) {
    float ms = 0.f;
    cudaEventElapsedTime(&ms, p.a, p.b);
    s->kstats[p.stat].ms += ms;
    s->kstats[p.stat].launches += 1;
    s->ev_pool.push_back(p.a);
    s->ev_pool.push_back(p.b);
  }
  s->pending.clear();
  return FSIM_OK;
}

int ensure_particle_capacity(fsim_sim* s, int64_t n) {
  if (n <= s->cap_p) return FSIM_OK;
  if (n > int64_t(0xFFFFFFF0u))
    return fail(s, FSIM_ERR_CAPACITY, "more than 2^32 particles is not supported");
  int64_t cap = std::max<int64_t>(n, 1024);
  // existing particles (if any) are moved over
  float* np[2] = {nullptr, nullptr};
  uint32_t* nk[2] = {nullptr, nullptr};
  uint32_t* nv[2] = {nullptr, nullptr};
  int rc;
  for (int b = 0; b < 2; ++b) {
    if ((rc = dmalloc(s, &np[b], size_t(9) * cap))) return rc;
    if ((rc = dmalloc(s, &nk[b], size_t(cap)))) return rc;
    if ((rc = dmalloc(s, &nv[b], size_t(cap)))) return rc;
  }
  if (s->n_total > 0 && s->part[s->cur]) {
    for (int f = 0; f < 9; ++f)
      FSIM_CK(s, cudaMemcpyAsync(np[s->cur] + f * cap, s->part[s->cur] + f * s->cap_p,
                                 size_t(s->n_total) * sizeof(float), cudaMemcpyDeviceToDevice,
                                 s->stream));
    FSIM_CK(s, cudaMemcpyAsync(nk[0], s->keys[0], size_t(s->n_total) * 4, cudaMemcpyDeviceToDevice,
                               s->stream));
    FSIM_CK(s, cudaStreamSynchronize(s->stream));
  }
  for (int b = 0; b < 2; ++b) {
    dfree(s->part[b]);
    dfree(s->keys[b]);
    dfree(s->vals[b]);
    s->part[b] = np[b];
    s->keys[b] = nk[b];
    s->vals[b] = nv[b];
  }
  s->cap_p = cap;
  return FSIM_OK;
}

__global__ void k_aos_to_soa(const float* __restrict__ aos, float* __restrict__ soa, int64_t n,
                             int64_t cap, int field0) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int d = 0; d < 3; ++d) soa[(field0 + d) * cap + i] = aos[3 * i + d];
}

__global__ void k_soa_to_aos(const float* __restrict__ soa, float* __restrict__ aos, int64_t n,
                             int64_t cap, int field0) {
  int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= n) return;
#pragma unroll
  for (int d = 0; d < 3; ++d) aos[3 * i + d] = soa[(field0 + d) * cap + i];
}

float inv_speed_from(const fsim_sim* s, float v_inf) {
  // FlipSimulation::CFL: v = max(sqrt(0.5*gravity), v_inf), floored at 1e-2
  float v = float(std::fmax(std::sqrt(0.5 * double(s->cfg.gravity)), double(v_inf)));
  if (v < 1e-2) v = float(1e-2);
  return float(1.0 / double(v));
}

int read_vmax(fsim_sim* s, float* vmax) {
  FSIM_CK(s, cudaMemcpyAsync(s->h_cnt + 4, s->d_cnt + 4, sizeof(int64_t), cudaMemcpyDeviceToHost,
                             s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  uint32_t bits = uint32_t(uint64_t(s->h_cnt[4]) & 0xFFFFFFFFull);
  std::memcpy(vmax, &bits, 4);
  return FSIM_OK;
}

void reset_grid_flags(fsim_sim* s) {
  s->grid_valid = s->bc_applied = s->saved = s->div_valid = s->pres_valid = false;
  s->phi_valid = s->extrapolated = s->weight_valid = false;
}

int need_topology(fsim_sim* s) {
  if (!s->have_topology) return fail(s, FSIM_ERR_STATE, "no particles uploaded or seeded");
  return FSIM_OK;
}

int need_grid(fsim_sim* s) {
  if (!s->have_topology || !s->grid_valid)
    return fail(s, FSIM_ERR_STATE, "grid is empty: run TransferParticlesToGrid first");
  return FSIM_OK;
}

int after_sort(fsim_sim* s) {
  reset_grid_flags(s);
  return FSIM_OK;
}

}  // namespace

int grow_particle_capacity(fsim_sim* s, int64_t n) { return ensure_particle_capacity(s, n); }

int ensure_leaf_capacity(fsim_sim* s, int64_t n_gleaf, int64_t n_pleaf) {
  int rc;
  if (n_gleaf > s->cap_leaf) {
    int64_t cap = std::min<int64_t>(int64_t(s->lm.dense), std::max<int64_t>(n_gleaf * 5 / 4, 64));
    dfree(s->vel); dfree(s->vold); dfree(s->weight);
    dfree(s->vel_on); dfree(s->vold_on); dfree(s->marker); dfree(s->d_nbr);
    if ((rc = dmalloc(s, &s->vel, size_t(cap) * 1536))) return rc;
    if ((rc = dmalloc(s, &s->vold, size_t(cap) * 1536))) return rc;
    if ((rc = dmalloc(s, &s->weight, size_t(cap) * 1536))) return rc;
    if ((rc = dmalloc(s, &s->vel_on, size_t(cap) * 16))) return rc;
    if ((rc = dmalloc(s, &s->vold_on, size_t(cap) * 16))) return rc;
    if ((rc = dmalloc(s, &s->marker, size_t(cap) * 512))) return rc;
    if ((rc = dmalloc(s, &s->d_nbr, size_t(cap) * 27))) return rc;
    s->cap_leaf = cap;
  }
  // one slot past the particle leaves: the PCG's zeroed null slot
  if (n_pleaf + 1 > s->cap_pleaf) {
    int64_t cap = std::min<int64_t>(int64_t(s->lm.dense) + 1,
                                    std::max<int64_t>((int64_t(n_pleaf) + 1) * 5 / 4, 64));
    dfree(s->d_cell_range); dfree(s->d_leaf_range);
    dfree(s->div); dfree(s->pres); dfree(s->r); dfree(s->p[0]); dfree(s->p[1]);
    for (int b = 0; b < 2; ++b) { dfree(s->cgw[b]); dfree(s->cgs[b]); }
    dfree(s->flags); dfree(s->x64); dfree(s->r64); dfree(s->p64[0]); dfree(s->p64[1]);
    dfree(s->Ap64); dfree(s->b64); dfree(s->zface); dfree(s->zface64); dfree(s->zflags);
    const size_t n = size_t(cap) * 512;
    if ((rc = dmalloc(s, &s->d_cell_range, n))) return rc;
    if ((rc = dmalloc(s, &s->d_leaf_range, size_t(cap)))) return rc;
    if ((rc = dmalloc(s, &s->div, n))) return rc;
    if ((rc = dmalloc(s, &s->pres, n))) return rc;
    if ((rc = dmalloc(s, &s->r, n))) return rc;
    if ((rc = dmalloc(s, &s->p[0], n))) return rc;
    if ((rc = dmalloc(s, &s->p[1], n))) return rc;
    if ((rc = dmalloc(s, &s->flags, n))) return rc;
    if ((rc = dmalloc(s, &s->zface, size_t(cap) * 384))) return rc;
    if ((rc = dmalloc(s, &s->zflags, size_t(cap) * 128))) return rc;
    s->cap_pleaf = cap;
  }
  return FSIM_OK;
}

}  // namespace fsim

using namespace fsim;

extern "C" {

const char* fsim_version(void) { return "fsim-gb300 0.1 (sm_103a)"; }

const char* fsim_last_error(const fsim_t* sim) {
  if (!sim) return g_scene_err.empty() ? "null handle" : g_scene_err.c_str();
  return sim->err.c_str();
}

int fsim_create(const fsim_config* cfg, fsim_t** out) {
  if (!cfg || !out) return FSIM_ERR_INVALID;
  *out = nullptr;
  for (int a = 0; a < 3; ++a)
    if (cfg->global_dims[a] < 8 || cfg->global_dims[a] > 1024) return FSIM_ERR_INVALID;
  if (cfg->boundary != FSIM_BOUNDARY_BOX && cfg->boundary != FSIM_BOUNDARY_TANK)
    return FSIM_ERR_INVALID;
  if (cfg->nparticles_per_cell < 1 || cfg->nparticles_per_cell > 64) return FSIM_ERR_INVALID;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev <= 0) return FSIM_ERR_NO_DEVICE;
  if (cfg->device < 0 || cfg->device >= ndev) return FSIM_ERR_INVALID;
  fsim_sim* s = new (std::nothrow) fsim_sim();
  if (!s) return FSIM_ERR_CAPACITY;
  s->cfg = *cfg;
  s->dev = cfg->device;
  if (cudaSetDevice(s->dev) != cudaSuccess) { delete s; return FSIM_ERR_CUDA; }
  cudaDeviceGetAttribute(&s->num_sms, cudaDevAttrMultiProcessorCount, s->dev);
  s->max_blocks = std::max(1, s->num_sms) * 16;  // a multiple of 4: partial rows stay 16-byte aligned
  // FSIM_PCG_GRAPH=0 turns the graph loop off (host polling)
  if (const char* g = std::getenv("FSIM_PCG_GRAPH")) s->use_graphs = g[0] != '0';
  // FSIM_PCG_PDL=0: plain edges between the graph's kernel nodes (default:
  // programmatic edges, each kernel launching while its predecessor finishes)
  if (const char* c = std::getenv("FSIM_PCG_PDL")) s->use_pdl = c[0] != '0';
  // FSIM_PCG_ZDIRECT=0/1: z-face planes or direct reads (default: by system size)
  if (const char* c = std::getenv("FSIM_PCG_ZDIRECT")) s->zdirect = c[0] == '1' ? 1 : 0;
  // FSIM_PCG_TMA=1: the bulk-copy staged spmv (opt-in)
  if (const char* c = std::getenv("FSIM_PCG_TMA")) s->tma_spmv = c[0] == '1' ? 1 : 0;
  // FSIM_PCG_TMA_WITHHOLD=1 (tests): the first solve's bulk-copy spmv holds one
  // stage's flags copy back until its wait has given up
  if (const char* c = std::getenv("FSIM_PCG_TMA_WITHHOLD")) s->tma_withhold = c[0] == '1';
  if (const char* c = std::getenv("FSIM_PCG_RES_WITHHOLD")) s->res_withhold = c[0] == '1';
  // FSIM_PCG_PIPE=0: the unpipelined hot kernels
  if (const char* c = std::getenv("FSIM_PCG_PIPE")) s->use_pipe = c[0] != '0';
  // FSIM_PCG_CG1=1: fp32 solves by the single-reduction iteration (opt-in)
  if (const char* c = std::getenv("FSIM_PCG_CG1")) s->pcg_cg1 = c[0] == '1' ? 1 : 0;
  // FSIM_PCG_RES=0/1: fp32 solves never / wherever it fits by the on-chip
  // resident loop (default: by system size)
  if (const char* c = std::getenv("FSIM_PCG_RES")) s->pcg_res = c[0] == '1' ? 1 : 0;
  for (int a = 0; a < 3; ++a) {
    s->lm.n[a] = cfg->global_dims[a];
    s->lm.lmax[a] = cfg->global_dims[a] / 8;
    s->lm.R[a] = s->lm.lmax[a] / 8 + 2;
    s->solid.n[a] = cfg->global_dims[a];
  }
  s->lm.dense = uint32_t(s->lm.R[0]) * s->lm.R[1] * s->lm.R[2] * 512u;
  s->solid.boundary = cfg->boundary;
  s->solid.ncub = 0;
  int rc = FSIM_OK;
  auto bail = [&](int code) {
    fsim_destroy(s);
    return code;
  };
  if (cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking) != cudaSuccess)
    return bail(FSIM_ERR_CUDA);
  const uint32_t D = s->lm.dense;
  if ((rc = dmalloc(s, &s->d_flag, D))) return bail(rc);
  if ((rc = dmalloc(s, &s->d_slot, D))) return bail(rc);
  if ((rc = dmalloc(s, &s->d_scan, size_t(D) * 2))) return bail(rc);
  if ((rc = dmalloc(s, &s->d_leaf_id, D))) return bail(rc);
  if ((rc = dmalloc(s, &s->d_cnt, 16))) return bail(rc);
  if ((rc = dmalloc(s, &s->d_sc, 1))) return bail(rc);
  if ((rc = dmalloc(s, &s->d_part, size_t(s->max_blocks) * 4))) return bail(rc);
  if ((rc = dmalloc(s, &s->d_partf, size_t(s->max_blocks) * 16))) return bail(rc);
  if (cudaMallocHost(&s->h_cnt, 16 * sizeof(int64_t)) != cudaSuccess) return bail(FSIM_ERR_CUDA);
  if (cudaMallocHost(&s->h_sc, sizeof(PcgScalars)) != cudaSuccess) return bail(FSIM_ERR_CUDA);
  cudaMemsetAsync(s->d_cnt, 0, 16 * sizeof(int64_t), s->stream);
  cudaMemsetAsync(s->d_sc, 0, sizeof(PcgScalars), s->stream);
  if (cfg->max_particles > 0) {
    if ((rc = ensure_particle_capacity(s, cfg->max_particles))) return bail(rc);
  }
  if (cudaStreamSynchronize(s->stream) != cudaSuccess) return bail(FSIM_ERR_CUDA);
  *out = s;
  return FSIM_OK;
}

int fsim_destroy(fsim_t* s) {
  if (!s) return FSIM_OK;
  if (s->dev >= 0) cudaSetDevice(s->dev);
  if (s->stream) cudaStreamSynchronize(s->stream);
  for (int b = 0; b < 2; ++b) { dfree(s->part[b]); dfree(s->keys[b]); dfree(s->vals[b]); }
  dfree(s->sort_tmp); dfree(s->scan_tmp); dfree(s->keys64[0]); dfree(s->keys64[1]);
  if (s->src_tmp) cudaFree(s->src_tmp);
  dfree(s->d_flag); dfree(s->d_slot); dfree(s->d_scan); dfree(s->d_leaf_id); dfree(s->d_nbr);
  dfree(s->d_cell_range); dfree(s->d_leaf_range);
  dfree(s->vel); dfree(s->vold); dfree(s->weight); dfree(s->vel_on); dfree(s->vold_on);
  dfree(s->marker); dfree(s->div); dfree(s->pres); dfree(s->r); dfree(s->p[0]); dfree(s->p[1]);
  for (int b = 0; b < 2; ++b) { dfree(s->cgw[b]); dfree(s->cgs[b]); }
  dfree(s->flags); dfree(s->zface); dfree(s->zface64); dfree(s->zflags);
  dfree(s->x64); dfree(s->r64); dfree(s->p64[0]);
  dfree(s->p64[1]); dfree(s->Ap64); dfree(s->b64); dfree(s->d_sc); dfree(s->d_part);
  dfree(s->d_partf); dfree(s->d_cnt);
  if (s->dense_tmp.p) cudaFree(s->dense_tmp.p);
  if (s->h_cnt) cudaFreeHost(s->h_cnt);
  if (s->h_sc) cudaFreeHost(s->h_sc);
  for (auto& p : s->pending) { cudaEventDestroy(p.a); cudaEventDestroy(p.b); }
  for (auto e : s->ev_pool) cudaEventDestroy(e);
  if (s->io_stream) {
    cudaStreamSynchronize(s->io_stream);
    cudaStreamDestroy(s->io_stream);
  }
  if (s->ev_main) cudaEventDestroy(s->ev_main);
  for (auto e : s->ev_loop)
    if (e) cudaEventDestroy(e);
  if (s->ev_io) cudaEventDestroy(s->ev_io);
  dfree(s->io_stage);
  if (s->p2g_nodes) cudaFree(s->p2g_nodes);
  if (s->p2g_touch) cudaFree(s->p2g_touch);
  if (s->p2g_low) cudaFree(s->p2g_low);
  if (s->stream) cudaStreamDestroy(s->stream);
  delete s;
  return FSIM_OK;
}

int fsim_get_stream(fsim_t* s, void** stream) {
  if (!s || !stream) return FSIM_ERR_INVALID;
  *stream = s->stream;
  return FSIM_OK;
}

int fsim_synchronize(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}

int fsim_add_solid_cuboid(fsim_t* s, const int32_t lo[3], const int32_t hi[3]) {
  if (!s || !lo || !hi) return FSIM_ERR_INVALID;
  if (s->solid.ncub >= kMaxCuboids) return fail(s, FSIM_ERR_CAPACITY, "at most 32 solid cuboids");
  for (int a = 0; a < 3; ++a) {
    s->solid.lo[s->solid.ncub][a] = std::max(lo[a], -1);
    s->solid.hi[s->solid.ncub][a] = std::min(hi[a], s->lm.n[a]);
  }
  s->solid.ncub++;
  return FSIM_OK;
}

int fsim_seed_fluid(fsim_t* s, const fsim_seed_pass* passes, int32_t npasses, uint64_t seed) {
  if (!s || (npasses > 0 && !passes)) return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  // count first with the current capacity; seed_fluid fails with CAPACITY
  // when it does not fit, then grow and retry once.
  s->n_total = 0;
  s->n_live = 0;
  s->seed = seed;
  int rc = seed_fluid(s, passes, npasses, seed);
  if (rc == FSIM_ERR_CAPACITY) {
    const int64_t need = s->h_cnt[5];
    if ((rc = ensure_particle_capacity(s, need))) return rc;
    rc = seed_fluid(s, passes, npasses, seed);
  }
  if (rc) return rc;
  return after_sort(s);
}

int fsim_add_source(fsim_t* s, const fsim_source* src) {
  if (!s || !src) return FSIM_ERR_INVALID;
  if (s->sources.size() >= size_t(FSIM_MAX_SOURCES))
    return fail(s, FSIM_ERR_CAPACITY, "at most FSIM_MAX_SOURCES sources");
  if (src->velocity_oscillating && !(src->box_period != 0.f))
    return fail(s, FSIM_ERR_INVALID, "an oscillating velocity needs box_period != 0");
  s->sources.push_back(*src);
  return FSIM_OK;
}

int fsim_set_time(fsim_t* s, double t) {
  if (!s) return FSIM_ERR_INVALID;
  s->time = t;
  return FSIM_OK;
}

int fsim_get_time(fsim_t* s, double* t) {
  if (!s || !t) return FSIM_ERR_INVALID;
  *t = s->time;
  return FSIM_OK;
}

int fsim_add_contribution_from_sources(fsim_t* s, float t) {
  if (!s) return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  int rc = need_topology(s);
  if (rc) return rc;
  return add_source_particles(s, t);
}

int fsim_delete_fluid_in_sources(fsim_t* s, float t) {
  if (!s) return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  int rc = need_topology(s);
  if (rc) return rc;
  if (s->sources.empty()) return FSIM_OK;
  if ((rc = delete_in_sources(s, t))) return rc;
  s->deleted_outside = true;  // dead keys among the live ones until the next sort
  return FSIM_OK;
}

int fsim_perturb_velocities(fsim_t* s, float sigma, uint64_t seed) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_topology(s);
  if (rc) return rc;
  return perturb(s, sigma, seed);
}

int fsim_upload_particles(fsim_t* s, const float* pos, const float* vel, const float* gvel,
                          int64_t n) {
  if (!s || n < 0 || (n > 0 && (!pos || !vel || !gvel))) return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  int rc;
  s->n_total = 0;
  s->n_live = 0;
  if ((rc = ensure_particle_capacity(s, n))) return rc;
  // stage AoS in the spare particle buffer, then scatter to SoA
  float* stage = s->part[s->cur ^ 1];
  const float* src[3] = {pos, vel, gvel};
  for (int f = 0; f < 3; ++f) {
    if (n == 0) break;
    FSIM_CK(s, cudaMemcpyAsync(stage + size_t(f) * 3 * s->cap_p, src[f], size_t(n) * 12,
                               cudaMemcpyHostToDevice, s->stream));
    FSIM_LAUNCH(s, "aos_to_soa", k_aos_to_soa, unsigned((n + 255) / 256), 256, 0,
                stage + size_t(f) * 3 * s->cap_p, s->part[s->cur], n, s->cap_p, 3 * f);
  }
  s->n_total = n;
  if ((rc = launch_keys_from_positions(s, 0, 0.f))) return rc;
  int64_t invalid = 0;
  if ((rc = rebin_uploaded(s, &invalid))) return rc;
  if (invalid != 0) {
    s->n_total = 0;
    s->have_topology = false;
    return fail(s, FSIM_ERR_INVALID, "particle positions must lie in [0, N] per axis");
  }
  return after_sort(s);
}

int fsim_particle_count(fsim_t* s, int64_t* n) {
  if (!s || !n) return FSIM_ERR_INVALID;
  if (!s->deleted_outside) { *n = s->n_live; return FSIM_OK; }
  FSIM_CK(s, cudaMemcpyAsync(s->h_cnt + 6, s->d_cnt + 6, sizeof(int64_t), cudaMemcpyDeviceToHost,
                             s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  *n = s->n_live - s->h_cnt[6];
  return FSIM_OK;
}

int fsim_download_particles(fsim_t* s, float* pos, float* vel, float* gvel, int64_t capacity,
                            int64_t* n) {
  if (!s || !n) return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  int64_t cnt = 0;
  int rc = fsim_particle_count(s, &cnt);
  if (rc) return rc;
  *n = cnt;
  if (cnt > capacity) return fail(s, FSIM_ERR_CAPACITY, "download capacity too small");
  const int64_t nl = s->n_live;
  if (nl == 0) return FSIM_OK;
  float* stage = s->part[s->cur ^ 1];  // spare buffer: 9*cap floats
  float* outs[3] = {pos, vel, gvel};
  std::vector<uint32_t> keys;
  if (s->deleted_outside) {
    keys.resize(size_t(nl));
    FSIM_CK(s, cudaMemcpyAsync(keys.data(), s->keys[0], size_t(nl) * 4, cudaMemcpyDeviceToHost,
                               s->stream));
  }
  if (!s->deleted_outside) {
    // all three fields: convert into their own staging slices, copy, one sync
    for (int f = 0; f < 3; ++f) {
      if (!outs[f]) continue;
      float* st = stage + size_t(f) * 3 * s->cap_p;
      FSIM_LAUNCH(s, "soa_to_aos", k_soa_to_aos, unsigned((nl + 255) / 256), 256, 0,
                  s->part[s->cur], st, nl, s->cap_p, 3 * f);
      FSIM_CK(s, cudaMemcpyAsync(outs[f], st, size_t(nl) * 12, cudaMemcpyDeviceToHost,
                                 s->stream));
    }
    FSIM_CK(s, cudaStreamSynchronize(s->stream));
    return FSIM_OK;
  }
  for (int f = 0; f < 3; ++f) {
    if (!outs[f]) continue;
    FSIM_LAUNCH(s, "soa_to_aos", k_soa_to_aos, unsigned((nl + 255) / 256), 256, 0,
                s->part[s->cur], stage, nl, s->cap_p, 3 * f);
    {
      std::vector<float> tmp(size_t(nl) * 3);
      FSIM_CK(s, cudaMemcpyAsync(tmp.data(), stage, size_t(nl) * 12, cudaMemcpyDeviceToHost,
                                 s->stream));
      FSIM_CK(s, cudaStreamSynchronize(s->stream));
      int64_t w = 0;
      for (int64_t i = 0; i < nl; ++i) {
        if (keys[size_t(i)] == kDeadKey) continue;
        for (int d = 0; d < 3; ++d) outs[f][3 * w + d] = tmp[size_t(3 * i + d)];
        ++w;
      }
    }
  }
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}

int fsim_cfl(fsim_t* s, float* inv_speed) {
  if (!s || !inv_speed) return FSIM_ERR_INVALID;
  float vmax = 0.f;
  if (s->have_topology && s->grid_valid) {
    int rc = launch_cfl(s);
    if (rc) return rc;
    if ((rc = read_vmax(s, &vmax))) return rc;
  }
  *inv_speed = inv_speed_from(s, vmax);
  return FSIM_OK;
}

int fsim_move_particles(fsim_t* s, float dt) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_topology(s);
  if (rc) return rc;
  if ((rc = launch_keys_from_positions(s, 1, dt))) return rc;
  if ((rc = rebuild_topology(s))) return rc;
  return after_sort(s);
}

int fsim_clear_grid(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  reset_grid_flags(s);
  return FSIM_OK;
}

int fsim_transfer_particles_to_grid(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_topology(s);
  if (rc) return rc;
  reset_grid_flags(s);
  if ((rc = launch_p2g(s, false, 0.f))) return rc;
  s->grid_valid = true;
  s->weight_valid = true;
  return FSIM_OK;
}

int fsim_apply_boundary_conditions(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  if ((rc = launch_apply_bc(s))) return rc;
  s->bc_applied = true;
  return FSIM_OK;
}

int fsim_save_grid_velocities(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  if ((rc = launch_save_velocities(s))) return rc;
  s->saved = true;
  return FSIM_OK;
}

int fsim_delete_outside_particles(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_topology(s);
  if (rc) return rc;
  if (!s->deleted_outside) FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 6, 0, 8, s->stream));
  if ((rc = launch_delete_outside(s))) return rc;
  s->deleted_outside = true;
  return FSIM_OK;
}

int fsim_reinitialize_phi(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  s->phi_valid = true;
  return FSIM_OK;
}

int fsim_add_gravity(fsim_t* s, float dt) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  return launch_add_gravity(s, dt);
}

int fsim_compute_divergence(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  if ((rc = launch_divergence(s))) return rc;
  s->div_valid = true;
  return FSIM_OK;
}

int fsim_pcg_default_params(const fsim_t* s, fsim_pcg_params* p) {
  if (!s || !p) return FSIM_ERR_INVALID;
  std::memset(p, 0, sizeof(*p));
  p->mode = FSIM_PCG_ABSOLUTE;
  p->precision = FSIM_PREC_FP32;
  p->max_iterations = 1500;
  p->max_refinements = 8;
  const int volume = s->lm.n[0] * s->lm.n[1] * s->lm.n[2];
  p->threshold = double(float(volume) * float(0.5 * 1e-8));
  p->tolerance = 1e-5;
  p->inner_tolerance = 1e-2;
  return FSIM_OK;
}

int fsim_pcg_solve(fsim_t* s, const fsim_pcg_params* prm, fsim_pcg_stats* st) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  if (!s->div_valid) return fail(s, FSIM_ERR_STATE, "ComputeDivergence has not run");
  fsim_pcg_stats local;
  if (!st) st = &local;
  std::memset(st, 0, sizeof(*st));
  if ((rc = pcg_solve(s, prm, st))) return rc;
  s->pres_valid = true;
  return FSIM_OK;
}

int fsim_update_velocity_from_pressure(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  if (!s->pres_valid) return fail(s, FSIM_ERR_STATE, "pressure has not been solved");
  return launch_pressure_update(s, false);
}

int fsim_get_velocity_update(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  if ((rc = launch_velocity_update(s))) return rc;
  FSIM_CK(s, cudaMemcpyAsync(s->h_cnt + 3, s->d_cnt + 3, sizeof(int64_t), cudaMemcpyDeviceToHost,
                             s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  if (s->h_cnt[3] != 0)
    return fail(s, FSIM_ERR_STATE,
                "GetVelocityUpdate: a velocity face is active without a saved velocity");
  s->saved = true;
  return FSIM_OK;
}

int fsim_update_particles_from_grid(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = need_grid(s);
  if (rc) return rc;
  s->extrapolated = true;
  return launch_g2p(s);
}

namespace {

// fsim_step_host: the positions are final once the step has sorted and
// gathered the particles (G2P changes only vel and gvel), so they are
// converted to AoS and copied to the host on the I/O stream while the rest
// of the step runs.
int start_early_position_download(fsim_sim* s) {
  const int64_t nl = s->n_live;
  s->io_early_n = -1;
  if (nl > s->io_early_cap || nl == 0) return FSIM_OK;  // the final download handles it
  if (s->io_stage_cap < s->cap_p) {
    dfree(s->io_stage);
    int rc = dmalloc(s, &s->io_stage, size_t(s->cap_p) * 3);
    if (rc) return rc;
    s->io_stage_cap = s->cap_p;
  }
  FSIM_CK(s, cudaEventRecord(s->ev_main, s->stream));
  FSIM_CK(s, cudaStreamWaitEvent(s->io_stream, s->ev_main, 0));
  k_soa_to_aos<<<unsigned((nl + 255) / 256), 256, 0, s->io_stream>>>(s->part[s->cur], s->io_stage,
                                                                     nl, s->cap_p, 0);
  s->launches++;
  FSIM_CK(s, cudaGetLastError());
  FSIM_CK(s, cudaMemcpyAsync(s->io_early_pos, s->io_stage, size_t(nl) * 12, cudaMemcpyDeviceToHost,
                             s->io_stream));
  s->io_early_n = nl;
  return FSIM_OK;
}

int ensure_io_stream(fsim_sim* s) {
  if (s->io_stream) return FSIM_OK;
  FSIM_CK(s, cudaStreamCreateWithFlags(&s->io_stream, cudaStreamNonBlocking));
  FSIM_CK(s, cudaEventCreateWithFlags(&s->ev_main, cudaEventDisableTiming));
  FSIM_CK(s, cudaEventCreateWithFlags(&s->ev_io, cudaEventDisableTiming));
  return FSIM_OK;
}

// Upload with the velocity copy on the I/O stream: positions and PIC
// velocities (which the rebinning and the advection read) go first on the
// handle's stream; the velocity lands while they are binned and sorted, and
// the particle gather waits for it.
int upload_overlapped(fsim_sim* s, const float* pos, const float* vel, const float* gvel,
                      int64_t n) {
  int rc;
  s->n_total = 0;
  s->n_live = 0;
  if ((rc = ensure_particle_capacity(s, n))) return rc;
  float* stage = s->part[s->cur ^ 1];
  if (n > 0) {
    for (int f = 0; f < 3; f += 2) {  // pos, gvel
      const float* src = f == 0 ? pos : gvel;
      FSIM_CK(s, cudaMemcpyAsync(stage + size_t(f) * 3 * s->cap_p, src, size_t(n) * 12,
                                 cudaMemcpyHostToDevice, s->stream));
      // the velocity copy starts when the gvel copy is done: run at the same
      // time, the three copies would share the host link and delay the two
      // the rebinning and the advection need first
      if (f == 2) {
        FSIM_CK(s, cudaEventRecord(s->ev_main, s->stream));
        FSIM_CK(s, cudaStreamWaitEvent(s->io_stream, s->ev_main, 0));
      }
      FSIM_LAUNCH(s, "aos_to_soa", k_aos_to_soa, unsigned((n + 255) / 256), 256, 0,
                  stage + size_t(f) * 3 * s->cap_p, s->part[s->cur], n, s->cap_p, 3 * f);
    }
    FSIM_CK(s, cudaMemcpyAsync(stage + size_t(3) * s->cap_p, vel, size_t(n) * 12,
                               cudaMemcpyHostToDevice, s->io_stream));
    k_aos_to_soa<<<unsigned((n + 255) / 256), 256, 0, s->io_stream>>>(
        stage + size_t(3) * s->cap_p, s->part[s->cur], n, s->cap_p, 3);
    s->launches++;
    FSIM_CK(s, cudaGetLastError());
    FSIM_CK(s, cudaEventRecord(s->ev_io, s->io_stream));
    s->io_vel_pending = true;
  }
  s->n_total = n;
  if ((rc = launch_keys_from_positions(s, 0, 0.f))) return rc;
  int64_t invalid = 0;
  if ((rc = rebin_uploaded(s, &invalid))) return rc;
  if (invalid != 0) {
    s->n_total = 0;
    s->have_topology = false;
    return fail(s, FSIM_ERR_INVALID, "particle positions must lie in [0, N] per axis");
  }
  return after_sort(s);
}

}  // namespace

int fsim_step_host(fsim_t* s, float dt, const fsim_pcg_params* prm, const float* pos,
                   const float* vel, const float* gvel, int64_t n, float* out_pos, float* out_vel,
                   float* out_gvel, int64_t capacity, int64_t* n_out, fsim_step_stats* st) {
  if (!s || !prm || !n_out || n < 0 || (n > 0 && (!pos || !vel || !gvel)))
    return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  // the overlapped path needs the particle buffers fixed during the step and
  // no deletion after the sort: no sources, no tank boundary
  const bool overlap = s->sources.empty() && s->cfg.boundary != FSIM_BOUNDARY_TANK;
  int rc = FSIM_OK;
  if (!overlap) {
    if ((rc = fsim_upload_particles(s, pos, vel, gvel, n))) return rc;
    if ((rc = fsim_step(s, dt, prm, st))) return rc;
    return fsim_download_particles(s, out_pos, out_vel, out_gvel, capacity, n_out);
  }
  if ((rc = ensure_io_stream(s))) return rc;
  rc = upload_overlapped(s, pos, vel, gvel, n);
  if (rc == FSIM_OK) {
    s->io_early_pos = out_pos;
    s->io_early_cap = capacity;
    s->io_early_n = -1;
    rc = fsim_step(s, dt, prm, st);
    s->io_early_pos = nullptr;
  }
  if (rc != FSIM_OK) {
    cudaStreamSynchronize(s->io_stream);
    s->io_vel_pending = false;
    return rc;
  }
  // velocities after G2P; positions unless the early copy took them
  const int64_t nl = s->n_live;
  *n_out = nl;
  if (nl > capacity) {
    cudaStreamSynchronize(s->io_stream);
    return fail(s, FSIM_ERR_CAPACITY, "download capacity too small");
  }
  float* stage = s->part[s->cur ^ 1];
  float* outs[3] = {s->io_early_n == nl ? nullptr : out_pos, out_vel, out_gvel};
  cudaError_t e = cudaSuccess;
  for (int f = 0; f < 3 && nl > 0 && e == cudaSuccess; ++f) {
    if (!outs[f]) continue;
    float* sg = stage + size_t(f) * 3 * s->cap_p;
    {
      fsim::ProfScope ps(s, "soa_to_aos");
      k_soa_to_aos<<<unsigned((nl + 255) / 256), 256, 0, s->stream>>>(s->part[s->cur], sg, nl,
                                                                     s->cap_p, 3 * f);
      s->launches++;
      e = cudaGetLastError();
    }
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(outs[f], sg, size_t(nl) * 12, cudaMemcpyDeviceToHost, s->stream);
  }
  // both streams finish before returning, also on an error: the early
  // position copy writes into the caller's buffer
  const cudaError_t e1 = cudaStreamSynchronize(s->stream);
  const cudaError_t e2 = cudaStreamSynchronize(s->io_stream);
  s->io_early_n = -1;
  if (e == cudaSuccess) e = e1;
  if (e == cudaSuccess) e = e2;
  if (e != cudaSuccess) return cuda_fail(s, e, "fsim_step_host download");
  return FSIM_OK;
}

int fsim_step(fsim_t* s, float dt, const fsim_pcg_params* prm, fsim_step_stats* st) {
  if (!s || !prm) return FSIM_ERR_INVALID;
  int rc = need_topology(s);
  if (rc) return rc;
  const float t = float(s->time);  // advanced_time_ (T = float)
  if (!s->sources.empty()) {
    // AddContributionFromSources(t); DeleteFluidInSources(t) is applied by
    // the advection kernel right after the move
    if ((rc = add_source_particles(s, t))) return rc;
    s->delete_in_sources = true;
    s->src_time = t;
  }
  // MoveParticles + DeleteParticlesInSolids.  The rebinning gather leaves
  // gvel behind: G2P below rewrites it for every live particle, and nothing
  // reads it before.  Not under the tank boundary, whose deletions after P2G
  // leave dead particles that G2P skips.
  if ((rc = launch_keys_from_positions(s, 1, dt))) return rc;
  s->gather_skip_gvel = s->cfg.boundary != FSIM_BOUNDARY_TANK;
  rc = rebuild_topology(s);
  s->gather_skip_gvel = false;
  if (rc) return rc;
  if (s->io_early_pos && (rc = start_early_position_download(s))) return rc;
  reset_grid_flags(s);
  // TransferParticlesToGrid + BC + SaveGridVelocities + AddGravity + BC
  if ((rc = launch_p2g(s, true, dt))) return rc;
  s->grid_valid = s->bc_applied = s->saved = s->phi_valid = true;
  if (s->cfg.boundary == FSIM_BOUNDARY_TANK) {
    FSIM_CK(s, cudaMemsetAsync(s->d_cnt + 6, 0, 8, s->stream));
    if ((rc = launch_delete_outside(s))) return rc;
    s->deleted_outside = true;
  }
  if ((rc = launch_divergence(s))) return rc;
  s->div_valid = true;
  fsim_pcg_stats ps;
  std::memset(&ps, 0, sizeof(ps));
  if ((rc = pcg_solve(s, prm, &ps))) return rc;
  s->pres_valid = true;
  if ((rc = launch_pressure_update(s, true))) return rc;
  s->extrapolated = true;
  if ((rc = launch_g2p(s))) return rc;
  float vmax = 0.f;
  if ((rc = read_vmax(s, &vmax))) return rc;
  if (st) {
    std::memset(st, 0, sizeof(*st));
    int64_t cnt = 0;
    if ((rc = fsim_particle_count(s, &cnt))) return rc;
    st->particles = cnt;
    st->particle_leaves = s->n_pleaf;
    st->grid_leaves = s->n_gleaf;
    st->pcg = ps;
    st->next_inv_speed = inv_speed_from(s, vmax);
  }
  s->time = double(t + dt);  // AdvanceTime, in T = float
  if (ps.status == FSIM_ERR_BREAKDOWN)
    return fail(s, FSIM_ERR_BREAKDOWN, "PCG breakdown: alpha or beta exceeded 1e5");
  return FSIM_OK;
}

int fsim_run_frames(fsim_t* s, int32_t nframes, float frame_rate, int32_t cfl,
                    const fsim_pcg_params* prm, fsim_frame_fn on_frame, void* user,
                    fsim_run_stats* st) {
  if (!s || !prm || nframes < 0 || !(frame_rate > 0.f) || cfl < 1) return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  fsim_run_stats acc;
  std::memset(&acc, 0, sizeof(acc));
  const float frame_step = 1.0f / frame_rate;  // params_.frame_step = T(1)/T(frame_rate)
  float inv = 0.f;
  int rc = fsim_cfl(s, &inv);
  if (rc) return rc;
  for (int f = 0; f < nframes; ++f) {
    float step = 0.f;  // ResetDt
    while (double(step) + 1e-5 < double(frame_step)) {
      float dt = 0.f;
      fsim_compute_dt(inv, cfl, frame_step, &step, &dt);
      fsim_step_stats ss;
      if ((rc = fsim_step(s, dt, prm, &ss))) return rc;
      inv = ss.next_inv_speed;
      acc.steps += 1;
      acc.pcg_iterations += ss.pcg.iterations;
      acc.last_dt = dt;
    }
    acc.frames += 1;
    if (on_frame) on_frame(s, f, user);
  }
  acc.time = s->time;
  if (st) *st = acc;
  return FSIM_OK;
}

int fsim_compute_dt(float inv_speed, int32_t cfl, float frame_step, float* time_in_frame,
                    float* dt_out) {
  if (!time_in_frame || !dt_out || !(frame_step > 0.f)) return FSIM_ERR_INVALID;
  // FlipDriver::WhileAndComputeDt for one partition
  float local_dt = float(cfl) * inv_speed;
  float dt = float(1.0 / double(frame_step));
  dt = (local_dt < dt) ? local_dt : dt;
  if (dt < frame_step / 10) dt = frame_step / 10;
  const float step = *time_in_frame;
  if (step + dt > frame_step) dt = frame_step - step;
  if (double(step + dt) > 0.9 * double(frame_step)) dt = frame_step - step;
  *time_in_frame = step + dt;
  *dt_out = dt;
  return FSIM_OK;
}

int fsim_download_field(fsim_t* s, int32_t field, float* out, uint8_t* active) {
  if (!s || !out) return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  return download_dense(s, field, out, active);
}

int fsim_download_marker(fsim_t* s, int32_t* out, uint8_t* active) {
  if (!s || !out) return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  return download_marker(s, out, active);
}

int fsim_download_leaves(fsim_t* s, int32_t* origins, int64_t capacity, int64_t* n) {
  if (!s || !n) return FSIM_ERR_INVALID;
  *n = s->have_topology ? s->n_pleaf : 0;
  if (*n > capacity) return fail(s, FSIM_ERR_CAPACITY, "leaf capacity too small");
  if (*n == 0) return FSIM_OK;
  std::vector<int32_t> ids(static_cast<size_t>(*n));
  FSIM_CK(s, cudaMemcpyAsync(ids.data(), s->d_leaf_id, size_t(*n) * 4, cudaMemcpyDeviceToHost,
                             s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  for (int64_t i = 0; i < *n; ++i) {
    int lx, ly, lz;
    leaf_coords(s->lm, uint32_t(ids[size_t(i)]), lx, ly, lz);
    origins[3 * i] = lx * 8;
    origins[3 * i + 1] = ly * 8;
    origins[3 * i + 2] = lz * 8;
  }
  return FSIM_OK;
}

int fsim_set_profiling(fsim_t* s, int32_t enabled) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = resolve_profile(s);
  s->profiling = enabled != 0;
  return rc;
}

int fsim_get_kernel_times(fsim_t* s, const char** names, double* total_ms, int64_t* launches,
                          int32_t capacity, int32_t* count) {
  if (!s || !count) return FSIM_ERR_INVALID;
  int rc = resolve_profile(s);
  if (rc) return rc;
  *count = int32_t(s->kstats.size());
  for (int32_t i = 0; i < *count && i < capacity; ++i) {
    if (names) names[i] = s->kstats[size_t(i)].name;
    if (total_ms) total_ms[i] = s->kstats[size_t(i)].ms;
    if (launches) launches[i] = s->kstats[size_t(i)].launches;
  }
  return FSIM_OK;
}

int fsim_reset_kernel_times(fsim_t* s) {
  if (!s) return FSIM_ERR_INVALID;
  int rc = resolve_profile(s);
  s->kstats.clear();
  return rc;
}

int fsim_launch_count(fsim_t* s, int64_t* launches) {
  if (!s || !launches) return FSIM_ERR_INVALID;
  *launches = s->launches;
  return FSIM_OK;
}

}  // extern "C"
