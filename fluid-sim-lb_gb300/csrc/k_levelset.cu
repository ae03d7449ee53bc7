// k_levelset.cu -- particles to a narrow-band level set (headless).
//
// Restates the method of the reference's converter
// (projects/particles-to-levelset/convert.cc:80-156): every particle is a
// sphere of radius R voxels (voxel size 1, index space = world space), the
// level set is the signed distance min_p(|x - p| - R) at the voxel points,
// clamped to the narrow band [-w, w] (OpenVDB's ParticlesToLevelSet
// rasterizeSpheres), followed by mean-filter passes over the band
// (LevelSetFilter::mean: the average of the 3^3 neighbourhood).  OpenVDB
// re-normalises the band after each filter pass (LevelSetTracker); that PDE
// step is not restated -- the output is the filtered, re-clamped field.
// The .vdb file of the converter becomes a dense device field that the
// caller downloads (same layout as fsim_download_field).
#include <algorithm>
#include <cmath>
#include <vector>

#include "fsim_internal.cuh"

namespace fsim {
namespace {

// order-preserving map float <-> uint32 for atomicMin on signed floats
__device__ __forceinline__ unsigned f2o(float f) {
  const unsigned u = __float_as_uint(f);
  return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}
__device__ __forceinline__ float o2f(unsigned u) {
  return __uint_as_float((u & 0x80000000u) ? (u & 0x7FFFFFFFu) : ~u);
}

struct LsArgs {
  const float* part;
  int64_t cap, n;
  const uint32_t* keys;
  int n0, n1, n2;  // dense extents (N + 2)
  float radius, half_width;
  unsigned* phi;   // ordered bits, dense
};

// one thread per particle: every voxel point within R + w of it
__global__ void k_ls_splat(const __grid_constant__ LsArgs a) {
  const int64_t i = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (i >= a.n || a.keys[i] == kDeadKey) return;
  const float p[3] = {a.part[i], a.part[a.cap + i], a.part[2 * a.cap + i]};
  const float reach = __fadd_rn(a.radius, a.half_width);
  int lo[3], hi[3];
  const int ext[3] = {a.n0, a.n1, a.n2};
#pragma unroll
  for (int d = 0; d < 3; ++d) {
    lo[d] = max(int(ceilf(__fsub_rn(p[d], reach))), -1);
    hi[d] = min(int(floorf(__fadd_rn(p[d], reach))), ext[d] - 2);
  }
  for (int x = lo[0]; x <= hi[0]; ++x)
    for (int y = lo[1]; y <= hi[1]; ++y)
      for (int z = lo[2]; z <= hi[2]; ++z) {
        const float dx = __fsub_rn(float(x), p[0]), dy = __fsub_rn(float(y), p[1]),
                    dz = __fsub_rn(float(z), p[2]);
        const float d2 = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)),
                                   __fmul_rn(dz, dz));
        const float dist = __fsub_rn(__fsqrt_rn(d2), a.radius);
        if (dist >= a.half_width) continue;
        const int64_t o = (int64_t(x + 1) * a.n1 + (y + 1)) * a.n2 + (z + 1);
        atomicMin(&a.phi[o], f2o(dist));
      }
}

// ordered bits -> clamped float; band = |phi| < w
__global__ void k_ls_finish(const unsigned* __restrict__ bits, float* __restrict__ phi,
                            int64_t n, float w) {
  const int64_t o = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (o >= n) return;
  const float v = o2f(bits[o]);
  phi[o] = fminf(fmaxf(v, -w), w);
}

// one mean-filter pass: band voxels take the mean of their 3^3 neighbourhood
// (neighbours outside the dense box count as the outside value w)
__global__ void k_ls_mean(const float* __restrict__ in, float* __restrict__ out, int n0, int n1,
                          int n2, float w) {
  const int64_t o = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  const int64_t tot = int64_t(n0) * n1 * n2;
  if (o >= tot) return;
  const float c = in[o];
  if (!(fabsf(c) < w)) {
    out[o] = c;
    return;
  }
  const int x = int(o / (int64_t(n1) * n2)), y = int((o / n2) % n1), z = int(o % n2);
  float s = 0.f;
  for (int a = -1; a <= 1; ++a)
    for (int b = -1; b <= 1; ++b)
      for (int e = -1; e <= 1; ++e) {
        const int xx = x + a, yy = y + b, zz = z + e;
        float v = w;
        if (xx >= 0 && yy >= 0 && zz >= 0 && xx < n0 && yy < n1 && zz < n2)
          v = in[(int64_t(xx) * n1 + yy) * n2 + zz];
        s = __fadd_rn(s, v);
      }
  out[o] = fminf(fmaxf(__fdiv_rn(s, 27.0f), -w), w);
}

__global__ void k_fill_u32(unsigned* __restrict__ p, int64_t n, unsigned v) {
  const int64_t o = int64_t(blockIdx.x) * blockDim.x + threadIdx.x;
  if (o < n) p[o] = v;
}

int level_set(fsim_t* s, float radius, float half_width, int mean_iterations, unsigned* bits,
              float* f[2], int64_t tot, float* phi) {
  const int n0 = s->lm.n[0] + 2, n1 = s->lm.n[1] + 2, n2 = s->lm.n[2] + 2;
  const unsigned g = unsigned((tot + 255) / 256);
  // every voxel starts outside the band: the ordered bits of +inf
  FSIM_LAUNCH(s, "levelset_fill", k_fill_u32, g, 256, 0, bits, tot, 0xFF800000u);
  LsArgs a;
  a.part = s->part[s->cur];
  a.cap = s->cap_p;
  a.n = s->n_live;
  a.keys = s->keys[0];
  a.n0 = n0;
  a.n1 = n1;
  a.n2 = n2;
  a.radius = radius;
  a.half_width = half_width;
  a.phi = bits;
  FSIM_LAUNCH(s, "levelset_splat", k_ls_splat, unsigned(std::max<int64_t>((a.n + 255) / 256, 1)),
              256, 0, a);
  FSIM_LAUNCH(s, "levelset_finish", k_ls_finish, g, 256, 0, bits, f[0], tot, half_width);
  for (int it = 0; it < mean_iterations; ++it) {
    FSIM_LAUNCH(s, "levelset_mean", k_ls_mean, g, 256, 0, f[0], f[1], n0, n1, n2, half_width);
    std::swap(f[0], f[1]);
  }
  FSIM_CK(s, cudaMemcpyAsync(phi, f[0], size_t(tot) * 4, cudaMemcpyDeviceToHost, s->stream));
  FSIM_CK(s, cudaStreamSynchronize(s->stream));
  return FSIM_OK;
}
}  // namespace
}  // namespace fsim

using namespace fsim;

extern "C" int fsim_particles_to_level_set(fsim_t* s, float radius, float half_width,
                                           int32_t mean_iterations, float* phi,
                                           uint8_t* active) {
  if (!s || !phi || !(radius > 0.f) || !(half_width > 0.f) || mean_iterations < 0)
    return FSIM_ERR_INVALID;
  cudaSetDevice(s->dev);
  if (!s->have_topology) return fail(s, FSIM_ERR_STATE, "no particles uploaded or seeded");
  const int64_t tot = int64_t(s->lm.n[0] + 2) * (s->lm.n[1] + 2) * (s->lm.n[2] + 2);
  unsigned* bits = nullptr;
  float* f[2] = {nullptr, nullptr};
  cudaError_t e = cudaMalloc(&bits, size_t(tot) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&f[0], size_t(tot) * 4);
  if (e == cudaSuccess) e = cudaMalloc(&f[1], size_t(tot) * 4);
  int rc = e == cudaSuccess ? level_set(s, radius, half_width, mean_iterations, bits, f, tot, phi)
                            : cuda_fail(s, e, "level set buffers");
  cudaStreamSynchronize(s->stream);
  if (bits) cudaFree(bits);
  if (f[0]) cudaFree(f[0]);
  if (f[1]) cudaFree(f[1]);
  if (rc) return rc;
  if (active)
    for (int64_t o = 0; o < tot; ++o) active[o] = std::fabs(phi[o]) < half_width ? 1 : 0;
  return FSIM_OK;
}
