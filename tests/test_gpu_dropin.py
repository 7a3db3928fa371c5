"""The C++ drop-in (include/rti/device.hpp) runs on the GPU and gives the same
results as the same trace through the Python binding of the C ABI.

A small C++ program uses rti::device<float, particle, reflection> exactly as
rti's users do (set_points / set_normals / set_grid_spacing / set_x / set_y /
set_number_of_rays / run / get_mc_estimates / get_hit_cnts), for a particle
whose sticking comes from get_sticking_probability(), one with a constant
`rtg_sticking`, one with get_sticking_field(), and the constant one with the
multi-hit window deposit (set_multi_hit_window).  Every run also calls
set(power_cosine_direction_z(5)), which must leave the cosine source in place as
in the reference; the extension set_source_exponent(5) selects cos^5.  The
Python mirror (rti_gb300.device) is held to the same rule."""
import os
import subprocess

import numpy as np
import pytest

from rti_gb300 import scenes

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PROGRAM = r'''
#include <cstdio>
#include <fstream>
#include <string>
#include <vector>
#include "rti/device.hpp"

struct per_disc : rti::particle::i_particle<float> {
  float get_sticking_probability(RTCRay&, RTCHit& hit, rti::geo::meta_geometry<float>&, rti::rng::i_rng&,
                                 rti::rng::i_rng::i_state&) override {
    return hit.primID % 2 ? 0.1f : 0.3f;
  }
  void init_new() override {}
};
struct constant : per_disc { static constexpr float rtg_sticking = 0.1f; };
struct field : per_disc {
  std::vector<float> get_sticking_field() { return std::vector<float>(N, 0.25f); }
  static size_t N;
};
size_t field::N = 0;

template <typename T>
std::vector<T> load(const std::string& path, size_t n) {
  std::vector<T> v(n);
  std::ifstream f(path, std::ios::binary);
  f.read(reinterpret_cast<char*>(v.data()), (std::streamsize)(n * sizeof(T)));
  return v;
}

template <typename P, typename R>
void run(const std::string& dir, const std::string& tag, size_t n, bool window = false, float exponent = 0) {
  auto pts = load<std::array<float, 3>>(dir + "/points.bin", n);
  auto nrm = load<std::array<float, 3>>(dir + "/normals.bin", n);
  auto rad = load<float>(dir + "/radii.bin", n);
  rti::device<float, P, R> d;
  d.set_points(pts);
  d.set_normals(nrm);
  d.set_grid_spacing(rad);
  d.set_x(rti::geo::bound_condition::PERIODIC);
  d.set_y(rti::geo::bound_condition::PERIODIC);
  d.set_number_of_rays(200000);
  if (window) d.set_multi_hit_window(5.0f);
  // rti's set() leaves the cosine source in place: the flux must not change
  rti::ray::power_cosine_direction_z<float> cos5(5.0f);
  d.set(cos5);
  if (exponent > 0) d.set_source_exponent(exponent);
  d.run();
  auto est = d.get_mc_estimates();
  auto cnt = d.get_hit_cnts();
  auto val = d.get_values();
  std::ofstream(dir + "/" + tag + "_est.bin", std::ios::binary)
      .write(reinterpret_cast<const char*>(est.data()), (std::streamsize)(est.size() * sizeof(float)));
  std::vector<unsigned long long> c(cnt.begin(), cnt.end());
  std::ofstream(dir + "/" + tag + "_cnt.bin", std::ios::binary)
      .write(reinterpret_cast<const char*>(c.data()), (std::streamsize)(c.size() * 8));
  std::ofstream(dir + "/" + tag + "_val.bin", std::ios::binary)
      .write(reinterpret_cast<const char*>(val.data()), (std::streamsize)(val.size() * 8));
}

int main(int argc, char** argv) {
  const std::string dir = argv[1];
  const size_t n = std::stoul(argv[2]);
  field::N = n;
  run<per_disc, rti::reflection::diffuse<float>>(dir, "per_disc", n);
  run<constant, rti::reflection::mixed<float, 10>>(dir, "constant", n);
  run<field, rti::reflection::specular<float>>(dir, "field", n);
  run<constant, rti::reflection::diffuse<float>>(dir, "window", n, true);
  run<constant, rti::reflection::diffuse<float>>(dir, "cos5", n, false, 5.0f);
  std::printf("ok\n");
  return 0;
}
'''


def test_cpp_dropin_matches_binding(rtg_lib, tmp_path):
    from rti_gb300 import _lib as L
    from rti_gb300.engine import device_run
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)
    n = t.n
    t.points.astype(np.float32).tofile(tmp_path / "points.bin")
    t.normals.astype(np.float32).tofile(tmp_path / "normals.bin")
    t.radii.astype(np.float32).tofile(tmp_path / "radii.bin")
    src = tmp_path / "use.cpp"
    src.write_text(PROGRAM)
    exe = tmp_path / "use"
    lib_dir = os.path.join(ROOT, "rti_gb300")
    r = subprocess.run(["g++", "-std=c++17", "-O1", "-I", os.path.join(ROOT, "include"), str(src), "-L", lib_dir,
                        "-lrtg", f"-Wl,-rpath,{lib_dir}", "-o", str(exe)], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    r = subprocess.run([str(exe), str(tmp_path), str(n)], capture_output=True, text=True)
    assert r.returncode == 0 and "ok" in r.stdout, r.stderr

    def expect(sticking_field, reflection, specular_fraction, sticking=0.1, exponent=1.0):
        c = L.default_config()
        c.source_exponent = exponent
        c.x_bound = c.y_bound = L.RTG_BOUND_PERIODIC
        c.reflection = reflection
        c.specular_fraction = specular_fraction
        c.sticking = sticking
        return device_run(t.points, t.normals, t.radii, n_rays=200000, seed=0, config=c,
                          sticking_field=sticking_field)

    def expect_window():
        from rti_gb300 import Engine
        e = Engine(0)
        e.upload_discs(t.points, t.normals, t.radii)
        e.configure(x_bound=L.RTG_BOUND_PERIODIC, y_bound=L.RTG_BOUND_PERIODIC, sticking=0.1, reset=True)
        e.set_deposit_mode(L.RTG_DEPOSIT_WINDOW, 5.0)
        e.trace(200000, 0)
        out = e.mc_estimates(), e.hit_counts()
        e.close()
        return out

    ids = np.arange(n)
    cases = {"per_disc": expect(np.where(ids % 2 == 1, 0.1, 0.3).astype(np.float32), L.RTG_REFLECT_DIFFUSE, 0.0),
             "constant": expect(None, L.RTG_REFLECT_MIXED, np.float32(0.1)),
             "field": expect(np.full(n, 0.25, np.float32), L.RTG_REFLECT_SPECULAR, 1.0),
             "window": expect_window(),
             "cos5": expect(None, L.RTG_REFLECT_DIFFUSE, 0.0, exponent=5.0)}
    for tag, (est, cnt) in cases.items():
        est_cpp = np.fromfile(tmp_path / f"{tag}_est.bin", dtype=np.float32)
        cnt_cpp = np.fromfile(tmp_path / f"{tag}_cnt.bin", dtype=np.uint64)
        val_cpp = np.fromfile(tmp_path / f"{tag}_val.bin", dtype=np.float64)
        assert np.array_equal(cnt_cpp, cnt), tag
        np.testing.assert_allclose(est_cpp, est, rtol=1e-6, atol=0, err_msg=tag)
        assert cnt_cpp.sum() > 0 and val_cpp.sum() > 0


def test_python_mirror_set_direction_keeps_cosine(rtg_lib):
    from rti_gb300 import device as D
    t = scenes.trench_discs(domain=1.2, width=0.4, depth=1.0)

    def run(setup):
        d = D.Device(D.ConstantSticking(0.1))
        d.set_points(t.points)
        d.set_normals(t.normals)
        d.set_grid_spacing(t.radii)
        d.set_x(D.BoundCondition.PERIODIC)
        d.set_y(D.BoundCondition.PERIODIC)
        d.set_number_of_rays(100000)
        setup(d)
        d.run()
        return d.get_hit_cnts()

    base = run(lambda d: None)
    assert np.array_equal(run(lambda d: d.set(D.PowerCosineDirectionZ(5.0))), base)
    cos5 = run(lambda d: d.set_source_exponent(5.0))
    assert not np.array_equal(cos5, base)
