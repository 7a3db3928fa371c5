// rtg_cli.cpp -- command-line driver on the C ABI, in place of rti's `rti`
// executable (rti src/rti/main/dev.cpp:136-288, options :51-99).
//
//   rtg --infile surface.vtp [--outfile out.vtp] [--number-of-rays N]
//       [--sticking S] [--triangles | --discs] [--seed K] [--device D]
//       [--ray-log N]
//
// As dev.cpp: the surface is read from a VTK XML file, the x/y box spans the
// disc centres and is periodic on both axes, the source plane lies at the
// highest centre + the largest radius (point_cloud_disc_geometry.hpp:84-87),
// cosine source, diffuse re-emission, constant sticking (default 0.8; a value
// outside (0, 1] is reset to 1 with a warning), 128 * 1024 rays by default.
// The output file gets rti's cell arrays and the metadata running-time[ns],
// git-hash, cmd and geo-name, plus `<name>.bounding-box.vtp` with the four
// side walls of the box as triangles.  Differences: --triangles traces a
// triangle mesh (dev.cpp rejects it); --max-threads and --single-hit are
// accepted and ignored (the GPU sets its own parallelism; dev.cpp parses
// --single-hit without using it).  --ray-log N writes raylog.vtp with every
// segment of the paths of the first N source rays (what dev.cpp writes when
// rti is compiled with RAYLOG_ON, ray_logger.hpp:23-71; their segment-0
// origins are RAYSRCLOG's source points).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <vector>

#include "rtg.h"

namespace {

struct Options {
  std::string infile, outfile;
  unsigned long long rays = 128ull * 1024ull;
  std::string sticking_text;
  bool triangles = false;
  unsigned long long seed = 0;
  int device = 0;
  unsigned long long ray_log = 0;  // source rays whose segments go to raylog.vtp
};

void usage(const char* argv0) {
  std::printf(
      "usage: %s --infile|-i FILE.vtp [--outfile|-o FILE.vtp] [--number-of-rays|--n-rays|-r N]\n"
      "          [--sticking-coefficient|--sticking-c|--sticking|-s S] [--triangles|--discs]\n"
      "          [--seed K] [--device D] [--max-threads|-m N] [--single-hit|--single] [--ray-log N]\n",
      argv0);
}

bool is(const char* a, std::initializer_list<const char*> names) {
  for (const char* n : names)
    if (std::strcmp(a, n) == 0) return true;
  return false;
}

bool parse(int argc, char** argv, Options& o) {
  for (int i = 1; i < argc; ++i) {
    const char* a = argv[i];
    auto value = [&](std::string& out) {
      if (i + 1 >= argc) return false;
      out = argv[++i];
      return true;
    };
    std::string v;
    if (is(a, {"--infile", "-i"})) {
      if (!value(o.infile)) return false;
    } else if (is(a, {"--outfile", "-o"})) {
      if (!value(o.outfile)) return false;
    } else if (is(a, {"--number-of-rays", "--n-rays", "-r"})) {
      if (!value(v)) return false;
      try {
        o.rays = std::stoull(v);
      } catch (...) {
      }
    } else if (is(a, {"--sticking-coefficient", "--sticking-c", "--sticking", "-s"})) {
      if (!value(o.sticking_text)) return false;
    } else if (is(a, {"--max-threads", "-m"})) {
      if (!value(v)) return false;
    } else if (is(a, {"--triangles"})) {
      o.triangles = true;
    } else if (is(a, {"--discs"})) {
      o.triangles = false;
    } else if (is(a, {"--single-hit", "--single"})) {
    } else if (is(a, {"--seed"})) {
      if (!value(v)) return false;
      o.seed = std::strtoull(v.c_str(), nullptr, 10);
    } else if (is(a, {"--ray-log"})) {
      if (!value(v)) return false;
      o.ray_log = std::strtoull(v.c_str(), nullptr, 10);
    } else if (is(a, {"--device"})) {
      if (!value(v)) return false;
      o.device = std::atoi(v.c_str());
    } else {
      std::fprintf(stderr, "unknown option %s\n", a);
      return false;
    }
  }
  return !o.infile.empty();
}

std::string extension(const std::string& p) {
  const size_t slash = p.find_last_of('/');
  const size_t dot = p.find_last_of('.');
  if (dot == std::string::npos || (slash != std::string::npos && dot < slash)) return "";
  return p.substr(dot);
}

std::string git_hash() {
  std::string out;
  FILE* p = popen("git rev-parse HEAD 2>/dev/null", "r");
  if (!p) return out;
  char buf[128];
  while (std::fgets(buf, sizeof buf, p)) out += buf;
  pclose(p);
  return out;
}

int fail(rtg_context* ctx, const char* what) {
  std::fprintf(stderr, "%s: %s\n", what, ctx ? rtg_last_error(ctx) : "");
  return EXIT_FAILURE;
}

}  // namespace

int main(int argc, char** argv) {
  Options o;
  if (!parse(argc, argv, o)) {
    usage(argv[0]);
    return EXIT_FAILURE;
  }
  float sticking = 0.8f;
  try {
    if (!o.sticking_text.empty()) sticking = (float)std::stod(o.sticking_text);
  } catch (...) {
  }
  if (!(0 < sticking && sticking <= 1)) {
    std::printf("Warning: sticking coefficient has been reset to sane value.\n");
    sticking = 1.0f;
  }
  std::printf("sticking coefficient == %g\n", sticking);
  if (extension(o.infile) == ".vtk") {
    std::printf("Recognized \".vtk\" input file file extension. Please convert the input file to vtp (e.g., using "
                "Paraview) and rerun %s with the new file.\nterminating\n",
                argv[0]);
    return EXIT_FAILURE;
  }
  char err[512] = {0};
  std::vector<float> pts, nrm, rad, vtx;
  std::vector<uint32_t> idx;
  int64_t n = 0, nv = 0, nt = 0;
  if (!o.triangles) {
    if (rtg_read_point_cloud(o.infile.c_str(), &n, nullptr, nullptr, nullptr, err, sizeof err) != RTG_OK) {
      std::fprintf(stderr, "cannot read %s: %s\n", o.infile.c_str(), err);
      return EXIT_FAILURE;
    }
    pts.resize(3 * n);
    nrm.resize(3 * n);
    rad.resize(n);
    if (rtg_read_point_cloud(o.infile.c_str(), &n, pts.data(), nrm.data(), rad.data(), err, sizeof err) != RTG_OK) {
      std::fprintf(stderr, "cannot read %s: %s\n", o.infile.c_str(), err);
      return EXIT_FAILURE;
    }
  } else {
    if (rtg_read_triangles(o.infile.c_str(), &nv, nullptr, &nt, nullptr, err, sizeof err) != RTG_OK) {
      std::fprintf(stderr, "cannot read %s: %s\n", o.infile.c_str(), err);
      return EXIT_FAILURE;
    }
    vtx.resize(3 * nv);
    idx.resize(3 * nt);
    if (rtg_read_triangles(o.infile.c_str(), &nv, vtx.data(), &nt, idx.data(), err, sizeof err) != RTG_OK) {
      std::fprintf(stderr, "cannot read %s: %s\n", o.infile.c_str(), err);
      return EXIT_FAILURE;
    }
  }
  // the box of dev.cpp: centre (vertex) extents, top at max z + max radius
  float lo[3] = {1e30f, 1e30f, 1e30f}, hi[3] = {-1e30f, -1e30f, -1e30f}, rmax = 0.0f;
  const std::vector<float>& P = o.triangles ? vtx : pts;
  for (size_t i = 0; i < P.size() / 3; ++i)
    for (int a = 0; a < 3; ++a) {
      lo[a] = std::min(lo[a], P[3 * i + a]);
      hi[a] = std::max(hi[a], P[3 * i + a]);
    }
  for (float r : rad) rmax = std::max(rmax, r);
  hi[2] = hi[2] + rmax;
  if (!(lo[0] < hi[0] && lo[1] < hi[1])) {
    std::fprintf(stderr, "degenerate x/y extent of the surface\n");
    return EXIT_FAILURE;
  }

  rtg_context* ctx = nullptr;
  if (rtg_create(&ctx, o.device) != RTG_OK) return fail(nullptr, "no usable CUDA device");
  std::unique_ptr<rtg_context, int (*)(rtg_context*)> guard(ctx, rtg_destroy);
  const int up = o.triangles ? rtg_upload_triangles(ctx, vtx.data(), idx.data(), nv, nt)
                             : rtg_upload_discs(ctx, pts.data(), nrm.data(), rad.data(), n);
  if (up != RTG_OK) return fail(ctx, "upload");
  rtg_config cfg;
  rtg_config_default(&cfg);
  cfg.x_bound = cfg.y_bound = RTG_BOUND_PERIODIC;
  cfg.reflection = RTG_REFLECT_DIFFUSE;
  cfg.sticking = sticking;
  cfg.source_exponent = 1.0f;
  cfg.box_mode = RTG_BOX_EXPLICIT;
  for (int a = 0; a < 3; ++a) {
    cfg.box_lo[a] = lo[a];
    cfg.box_hi[a] = hi[a];
  }
  if (rtg_set_config(ctx, &cfg) != RTG_OK) return fail(ctx, "configuration");
  // room for long paths: 2^16 segments per logged ray, at most 2^26 records
  if (o.ray_log > 0 &&
      rtg_set_segment_log(ctx, 0, o.ray_log, std::min<unsigned long long>(o.ray_log << 16, 1ull << 26)) != RTG_OK)
    return fail(ctx, "ray log");
  if (rtg_trace(ctx, o.rays, o.seed, nullptr) != RTG_OK) return fail(ctx, "trace");
  rtg_tally t;
  if (rtg_get_tally(ctx, &t) != RTG_OK) return fail(ctx, "trace");
  const char* geo = o.triangles ? "triangles" : "discs";
  std::printf("===[rtg]=== %s %s %llurays %gseconds (%llu hits, %llu misses, %llu segments)\n", geo,
              o.infile.c_str(), (unsigned long long)t.num_rays, t.trace_ms * 1e-3, (unsigned long long)t.hitc,
              (unsigned long long)t.nonhitc, (unsigned long long)t.segments);

  if (o.ray_log > 0) {
    std::printf("Writing ray log to raylog.vtp\n");
    if (rtg_write_segment_log_vtp(ctx, "raylog.vtp") != RTG_OK) return fail(ctx, "ray log");
  }
  if (!o.outfile.empty()) {
    if (extension(o.outfile) != ".vtp") {
      std::printf("Appending .vtp to the given file name\n");
      o.outfile += ".vtp";
    }
    std::string cmd;
    for (int i = 0; i < argc; ++i) (cmd += " ") += argv[i];
    char ns[64];
    std::snprintf(ns, sizeof ns, "%llu", (unsigned long long)(t.trace_ms * 1e6));
    const std::string hash = git_hash();
    const char* keys[] = {"running-time[ns]", "git-hash", "cmd", "geo-name"};
    const char* vals[] = {ns, hash.c_str(), cmd.c_str(), geo};
    std::printf("Writing output to %s\n", o.outfile.c_str());
    if (rtg_write_vtp(ctx, o.outfile.c_str(), keys, vals, 4) != RTG_OK) return fail(ctx, "write");
    // the side walls of the periodic box (boundary_x_y), two triangles each
    const std::string bb = o.outfile.substr(0, o.outfile.size() - 4) + ".bounding-box.vtp";
    const float z0 = lo[2], z1 = hi[2];
    const float bv[8 * 3] = {lo[0], lo[1], z0, hi[0], lo[1], z0, hi[0], hi[1], z0, lo[0], hi[1], z0,
                             lo[0], lo[1], z1, hi[0], lo[1], z1, hi[0], hi[1], z1, lo[0], hi[1], z1};
    const uint32_t bt[8 * 3] = {0, 1, 5, 0, 5, 4, 1, 2, 6, 1, 6, 5, 2, 3, 7, 2, 7, 6, 3, 0, 4, 3, 4, 7};
    std::printf("Writing bounding box to %s\n", bb.c_str());
    if (rtg_write_vtp_triangles(bb.c_str(), 8, bv, 8, bt, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                                nullptr, 0) != RTG_OK) {
      std::fprintf(stderr, "cannot write %s\n", bb.c_str());
      return EXIT_FAILURE;
    }
  }
  return EXIT_SUCCESS;
}
