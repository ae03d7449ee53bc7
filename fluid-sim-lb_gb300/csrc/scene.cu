// scene.cu -- init-file scenes: the reference's configuration parser and the
// scaling its driver applies at initialisation (host code).
//
// Restates FlipApp::ParseSimulationConfiguration (common/flip_app.cc:
// 159-251, tokens split on ", :" by GetTokens, :127-148), the defaults of
// SimulationConfiguration (common/flip_app.h:71-81, force (0,1,0) from
// flip_app.cc:101) and the part of FlipDriver::Initialize
// (common/flip_app_sim.cc:70-183) that turns the configuration into grid
// quantities: scaled gravity, forces, sources, solids and seeding passes.
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "fsim_internal.cuh"

namespace fsim {

thread_local std::string g_scene_err;

namespace {

std::vector<std::string> tokens_of(const std::string& line) {
  std::vector<std::string> t;
  size_t i = 0;
  const char* delim = ", :";
  while (i < line.size()) {
    while (i < line.size() && std::strchr(delim, line[i])) ++i;
    size_t j = i;
    while (j < line.size() && !std::strchr(delim, line[j])) ++j;
    if (j > i) t.emplace_back(line.substr(i, j - i));
    i = j;
  }
  return t;
}

struct Cursor {
  const std::vector<std::string>& t;
  size_t id;
  bool ok = true;
  float num() {
    if (id >= t.size()) { ok = false; return 0.f; }
    const char* s = t[id++].c_str();
    char* end = nullptr;
    const double v = std::strtod(s, &end);
    if (end == s) ok = false;
    return float(v);
  }
  int integer() { return int(num()); }
  void vec3(float v[3]) { for (int d = 0; d < 3; ++d) v[d] = num(); }
};

struct ParsedFluid {
  bool cube;
  float a[3], b[3], r, vel[3];
};

int bad(const std::string& msg) {
  g_scene_err = msg;
  return FSIM_ERR_INVALID;
}

}  // namespace
}  // namespace fsim

using namespace fsim;

extern "C" int fsim_scene_parse(const char* text, const int32_t dims[3], fsim_scene* out) {
  g_scene_err.clear();
  if (!text || !dims || !out) return bad("null argument");
  for (int d = 0; d < 3; ++d)
    if (dims[d] < 1) return bad("dims must be positive");
  std::memset(out, 0, sizeof(*out));
  // SimulationConfiguration defaults
  int fluid = 1, boundary = 0;
  float gravity = 9.8f, force[3] = {0.f, 1.f, 0.f};
  std::vector<ParsedFluid> fluids;
  std::vector<fsim_source> sources;
  std::vector<std::pair<std::vector<float>, int>> solids;  // start+end, line
  const std::string all(text);
  size_t pos = 0;
  int lineno = 0;
  while (pos <= all.size()) {
    size_t nl = all.find('\n', pos);
    if (nl == std::string::npos) nl = all.size();
    std::string line = all.substr(pos, nl - pos);
    pos = nl + 1;
    ++lineno;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    const std::vector<std::string> t = tokens_of(line);
    if (t.empty()) continue;
    const std::string& key = t[0];
    Cursor c{t, 1};
    const std::string where = " (line " + std::to_string(lineno) + ")";
    if (key == "fluid") {
      fluid = c.integer();
    } else if (key == "boundary") {
      boundary = c.integer();
    } else if (key == "gravity") {
      gravity = c.num();
    } else if (key == "force") {
      c.vec3(force);
    } else if (key == "fluid-cube" || key == "fluid-sphere") {
      ParsedFluid f;
      std::memset(&f, 0, sizeof(f));
      f.cube = key == "fluid-cube";
      c.vec3(f.a);
      if (f.cube) c.vec3(f.b); else f.r = c.num();
      c.vec3(f.vel);
      if (c.ok) fluids.push_back(f);
    } else if (key == "source-static" || key == "source-timed") {
      fsim_source s;
      std::memset(&s, 0, sizeof(s));
      c.vec3(s.lo);
      c.vec3(s.hi);
      c.vec3(s.velocity);
      if (key == "source-timed") {
        s.timed = 1;
        s.start_time = c.num();
        s.end_time = c.num();
      }
      if (c.ok) sources.push_back(s);
    } else if (key == "source-oscillating") {
      fsim_source s;
      std::memset(&s, 0, sizeof(s));
      c.vec3(s.lo);
      c.vec3(s.hi);
      c.vec3(s.lo2);
      c.vec3(s.hi2);
      s.box_period = c.num();
      c.vec3(s.velocity);
      c.vec3(s.velocity2);
      s.velocity_period = c.num();
      s.box_oscillating = 1;
      s.velocity_oscillating = 1;
      if (c.ok) sources.push_back(s);
    } else if (key == "solid") {
      std::vector<float> box(6);
      for (int k = 0; k < 6; ++k) box[size_t(k)] = c.num();
      if (c.ok) solids.emplace_back(box, lineno);
    } else {
      continue;  // not a configuration key
    }
    if (!c.ok) return bad("malformed '" + key + "' line" + where);
  }
  if (boundary < 0 || boundary > 1) return bad("boundary must be 0 (box) or 1 (tank)");
  if (fluid < 0 || fluid > 2) return bad("fluid must be 0, 1 or 2");
  const float N[3] = {float(dims[0]), float(dims[1]), float(dims[2])};
  // T scaled_gravity = config_.gravity * (T(global_dims[1])/128.0)
  const float sg = float(double(gravity) * (double(float(dims[1])) / 128.0));
  out->fluid = fluid;
  out->boundary = boundary;
  out->gravity = sg;
  for (int d = 0; d < 3; ++d) out->force[d] = force[d] * sg;
  // sources: ScaleBox(global_dims), ScaleVelocity(scaled_gravity)
  if (sources.size() > size_t(FSIM_MAX_SOURCES)) {
    g_scene_err = "more than 16 sources";
    return FSIM_ERR_CAPACITY;
  }
  for (size_t q = 0; q < sources.size(); ++q) {
    fsim_source s = sources[q];
    for (int d = 0; d < 3; ++d) {
      s.lo[d] *= N[d]; s.hi[d] *= N[d]; s.lo2[d] *= N[d]; s.hi2[d] *= N[d];
      s.velocity[d] *= sg; s.velocity2[d] *= sg;
    }
    out->sources[q] = s;
  }
  out->nsources = int32_t(sources.size());
  // solids: Cube::Scale, then Cube::get_coord_bbox (common/primitives.cc:36-53)
  if (solids.size() > size_t(FSIM_SCENE_MAX_SOLIDS)) {
    g_scene_err = "more than 32 solids";
    return FSIM_ERR_CAPACITY;
  }
  for (size_t q = 0; q < solids.size(); ++q) {
    float st[3], en[3];
    for (int d = 0; d < 3; ++d) {
      st[d] = solids[q].first[size_t(d)] * N[d];
      en[d] = solids[q].first[size_t(3 + d)] * N[d];
      const float tol = 1e-2f;
      if (!(st[d] <= tol + std::floor(st[d])) || !(std::ceil(en[d]) <= en[d] + tol))
        return bad("solid cube not on whole cells (line " +
                   std::to_string(solids[q].second) + ")");
    }
    for (int d = 0; d < 3; ++d) {
      int a = int(st[d]), b = int(en[d] - 1.f);  // Coord(start), Coord(end - 1)
      if (a > b) b = a;
      out->solid_lo[q][d] = a;
      out->solid_hi[q][d] = b;
    }
  }
  out->nsolids = int32_t(solids.size());
  // seeding passes: the preset, then the additional fluids
  std::vector<fsim_seed_pass> passes;
  if (fluid == 1) {
    // InitializeMultipleWaterDrops(height, {centre}, {radius})
    fsim_seed_pass p;
    std::memset(&p, 0, sizeof(p));
    p.nshapes = 2;
    p.shapes[0].kind = FSIM_SHAPE_POOL;
    p.shapes[0].a[1] = float(dims[1] / 4);
    p.shapes[1].kind = FSIM_SHAPE_SPHERE;
    p.shapes[1].a[0] = float(dims[0] / 2);
    p.shapes[1].a[1] = float(dims[1] * 3 / 4);
    p.shapes[1].a[2] = float(dims[2] * 5 / 8);
    p.shapes[1].r = float(double(float(dims[0] / 4)) * 0.8);
    passes.push_back(p);
  } else if (fluid == 2) {
    // InitializeWaterCuboid(Cube(0, (N0/4-1, N1*3/4-1, N2-1)), 0)
    fsim_seed_pass p;
    std::memset(&p, 0, sizeof(p));
    p.nshapes = 1;
    p.shapes[0].kind = FSIM_SHAPE_CUBOID;
    p.shapes[0].b[0] = float(dims[0] / 4) - 1.f;
    p.shapes[0].b[1] = float(dims[1] * 3 / 4) - 1.f;
    p.shapes[0].b[2] = float(dims[2]) - 1.f;
    passes.push_back(p);
  }
  for (const ParsedFluid& f : fluids) {
    fsim_seed_pass p;
    std::memset(&p, 0, sizeof(p));
    p.nshapes = 1;
    if (f.cube) {
      p.shapes[0].kind = FSIM_SHAPE_CUBOID;
      for (int d = 0; d < 3; ++d) {
        p.shapes[0].a[d] = f.a[d] * N[d];
        p.shapes[0].b[d] = f.b[d] * N[d] - 1.f;
      }
    } else {
      p.shapes[0].kind = FSIM_SHAPE_SPHERE;
      for (int d = 0; d < 3; ++d) p.shapes[0].a[d] = f.a[d] * N[d];
      p.shapes[0].r = f.r * N[0];
    }
    for (int d = 0; d < 3; ++d) p.velocity[d] = f.vel[d] * sg;
    passes.push_back(p);
  }
  if (passes.size() > 8) {
    g_scene_err = "more than 8 seeding passes";
    return FSIM_ERR_CAPACITY;
  }
  for (size_t q = 0; q < passes.size(); ++q) out->passes[q] = passes[q];
  out->npasses = int32_t(passes.size());
  return FSIM_OK;
}
