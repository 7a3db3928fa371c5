// rti/device.hpp -- drop-in for rti::device<numeric_type, particle_type,
// reflection_type> (rti: src/rti/device.hpp:34-297) on top of librtg's C ABI.
//
// Same template parameters, setters, defaults and getters as the reference:
// set_points / set_normals / set_grid_spacing (the spacing of a point is its
// disc radius, device.hpp:213-216) / set_number_of_rays (default 1024) /
// set_x / set_y (default REFLECTIVE) / set(direction), run(),
// get_mc_estimates() (normalised, neighbourhood-smoothed, device.hpp:154-187)
// and get_hit_cnts().  The trace runs on the GPU in librtg; link with -lrtg.
//
// Differences a caller can see:
//   * no Embree and no VTK: RTCRay / RTCHit below are plain structs with
//     Embree's field names so that existing particle classes compile;
//   * sticking comes from the particle type: `static constexpr rtg_sticking`
//     (one value), else a member get_sticking_field() (one value per disc),
//     else get_sticking_probability() called once per disc on the host
//     (normal-incidence ray, hit.primID = disc id) -- so a sticking that
//     depends on the incoming direction or on random state is evaluated at
//     normal incidence;
//   * reflection_type selects diffuse, specular or mixed re-emission
//     (rti::reflection::diffuse / specular / mixed below, or any type providing
//     `static constexpr int rtg_mode` and `static constexpr float
//     rtg_specular_fraction`);
//   * set(direction) changes nothing, as in the reference: there it assigns
//     through a reference member bound to the cosine source, which copies
//     only the (empty) i_direction base, so the cosine source stays
//     (device.hpp:77-80, 295-296).  A cos^n source is selected by the
//     extension set_source_exponent(n) instead;
//   * errors throw std::runtime_error with librtg's message, where the
//     reference asserts;
//   * extra getters: get_values() (raw S1 per disc, FP64), get_relative_error(),
//     get_vov().
#pragma once

#include <array>
#include <cstdint>
#include <cstring>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <vector>

#include "../rtg.h"

// Ray and hit records with Embree 3's member names (tracer.hpp:130).
struct RTCRay {
  float org_x, org_y, org_z, tnear;
  float dir_x, dir_y, dir_z, time;
  float tfar;
  unsigned int mask, id, flags;
};
struct RTCHit {
  float Ng_x, Ng_y, Ng_z;
  float u, v;
  unsigned int primID, geomID;
  unsigned int instID[1];
};

namespace rti {
namespace util {
template <typename T> using pair = std::array<T, 2>;
template <typename T> using triple = std::array<T, 3>;
template <typename T> using quadruple = std::array<T, 4>;
}  // namespace util

namespace geo {
enum class bound_condition { REFLECTIVE, PERIODIC };  // geo/bound_condition.hpp:4-6

template <typename Ty>
class meta_geometry {  // geo/meta_geometry.hpp:9-24 (the parts a particle may query)
 public:
  virtual ~meta_geometry() {}
  virtual util::triple<Ty> get_normal(unsigned int primID) = 0;
  virtual util::triple<Ty> get_new_origin(RTCRay& r, unsigned int) {
    return {(Ty)(r.org_x + r.dir_x * r.tfar), (Ty)(r.org_y + r.dir_y * r.tfar), (Ty)(r.org_z + r.dir_z * r.tfar)};
  }
};
}  // namespace geo

namespace rng {
class i_rng {  // rng/i_rng.hpp:11-30
 public:
  virtual ~i_rng() {}
  struct i_state {
    virtual ~i_state() {}
    virtual std::unique_ptr<i_state> clone() const = 0;
  };
  virtual uint64_t get(i_state& s) const = 0;
  virtual uint64_t min() const = 0;
  virtual uint64_t max() const = 0;
};

// A small host generator (splitmix64) handed to particle callbacks.
class splitmix_rng : public i_rng {
 public:
  struct state : i_state {
    uint64_t x = 0x9E3779B97F4A7C15ull;
    std::unique_ptr<i_state> clone() const override { return std::unique_ptr<i_state>(new state(*this)); }
  };
  uint64_t get(i_state& s) const override {
    uint64_t& x = static_cast<state&>(s).x;
    uint64_t z = (x += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
  }
  uint64_t min() const override { return 0; }
  uint64_t max() const override { return ~0ull; }
};
}  // namespace rng

namespace particle {
template <typename numeric_type>
class i_particle {  // particle/i_particle.hpp:9-16
 public:
  virtual ~i_particle() {}
  virtual numeric_type get_sticking_probability(RTCRay& rayin, RTCHit& hitin,
                                                geo::meta_geometry<numeric_type>& geometry, rng::i_rng& rng,
                                                rng::i_rng::i_state& rngstate) = 0;
  virtual void init_new() = 0;
};
}  // namespace particle

namespace reflection {
template <typename Ty>
class i_reflection {  // reflection/i_reflection.hpp:9-19 (selected by type, run on the GPU)
 public:
  virtual ~i_reflection() {}
};
template <typename Ty>
class diffuse : public i_reflection<Ty> {
 public:
  static constexpr int rtg_mode = RTG_REFLECT_DIFFUSE;
  static constexpr float rtg_specular_fraction = 0.0f;
};
template <typename Ty>
class specular : public i_reflection<Ty> {
 public:
  static constexpr int rtg_mode = RTG_REFLECT_SPECULAR;
  static constexpr float rtg_specular_fraction = 1.0f;
};
// Specular with probability SpecularPercent / 100, else diffuse (no
// counterpart in rti; the mixture of the hole benchmark).
template <typename Ty, int SpecularPercent>
class mixed : public i_reflection<Ty> {
  static_assert(0 <= SpecularPercent && SpecularPercent <= 100, "a percentage");

 public:
  static constexpr int rtg_mode = RTG_REFLECT_MIXED;
  static constexpr float rtg_specular_fraction = SpecularPercent / 100.0f;
};
}  // namespace reflection

namespace ray {
template <typename Ty>
class i_direction {  // ray/i_direction.hpp
 public:
  virtual ~i_direction() {}
  virtual Ty rtg_exponent() const = 0;
};
template <typename Ty>
class cosine_direction_z : public i_direction<Ty> {  // ray/cosine_direction_z.hpp
 public:
  Ty rtg_exponent() const override { return (Ty)1; }
};
template <typename Ty>
class power_cosine_direction_z : public i_direction<Ty> {  // ray/power_cosine_direction_z.hpp
 public:
  explicit power_cosine_direction_z(Ty e) : exp_(e) {}
  Ty rtg_exponent() const override { return exp_; }

 private:
  Ty exp_;
};
}  // namespace ray

namespace detail {
// particle_type::get_sticking_field() -> one sticking value per disc
template <typename P, typename = void>
struct has_sticking_field : std::false_type {};
template <typename P>
struct has_sticking_field<P, std::void_t<decltype(std::declval<P&>().get_sticking_field())>> : std::true_type {};
// particle_type::rtg_sticking -> one constant sticking for every disc
template <typename P, typename = void>
struct has_constant_sticking : std::false_type {};
template <typename P>
struct has_constant_sticking<P, std::void_t<decltype(P::rtg_sticking)>> : std::true_type {};
}  // namespace detail

using ::rti::geo::bound_condition;
using ::rti::particle::i_particle;
using ::rti::reflection::i_reflection;

template <typename numeric_type, typename particle_type, typename reflection_type>
class device final {
  static_assert(std::is_same<numeric_type, float>::value, "the engine traces in single precision");
  static_assert(std::is_base_of<i_particle<numeric_type>, particle_type>::value, "Precondition");
  static_assert(std::is_base_of<i_reflection<numeric_type>, reflection_type>::value, "Precondition");

 public:
  device() {}
  ~device() {}

  void set_points(std::vector<std::array<numeric_type, 3>> points_) { points = points_; }
  void set_normals(std::vector<std::array<numeric_type, 3>> normals_) { normals = normals_; }
  void set_grid_spacing(std::vector<numeric_type> spacing_) { spacing = spacing_; }
  void set_number_of_rays(size_t numofrays_) { numofrays = numofrays_; }
  void set_x(bound_condition cond) { xCond = cond; }
  void set_y(bound_condition cond) { yCond = cond; }
  // The reference's set() leaves its cosine source in place (an assignment
  // through a reference member that copies only the i_direction base); so
  // does this one, so that a simulator's flux does not change when it
  // switches to this header.
  void set(ray::i_direction<numeric_type>& srcDirection) { (void)srcDirection; }
  // Extension (no counterpart in the reference): the source emits with
  // density cos^n of the polar angle (power_cosine_direction_z), n >= 0;
  // default 1 (cosine_direction_z).
  void set_source_exponent(numeric_type n) { exponent = n; }
  void set_seed(uint64_t s) { seed = s; }
  void set_cuda_device(int d) { cuda_device = d; }
  // rti's other treatment of overlapping discs, the multi-hit window of
  // trace/point_cloud_context.hpp (rti: 5 radii), instead of its tracer's
  // neighbour deposit; radii < 0 selects the neighbour deposit again.
  void set_multi_hit_window(numeric_type radii = 5) { window = radii; }

  void run() {
    if (points.size() != spacing.size() || points.size() != normals.size())
      throw std::runtime_error("rti::device: points, normals and grid spacing differ in length");
    const size_t n = points.size();
    rtg_config cfg;
    rtg_config_default(&cfg);
    cfg.x_bound = xCond == bound_condition::PERIODIC ? RTG_BOUND_PERIODIC : RTG_BOUND_REFLECTIVE;
    cfg.y_bound = yCond == bound_condition::PERIODIC ? RTG_BOUND_PERIODIC : RTG_BOUND_REFLECTIVE;
    cfg.reflection = reflection_type::rtg_mode;
    cfg.specular_fraction = reflection_type::rtg_specular_fraction;
    cfg.source_exponent = (float)exponent;
    std::vector<float> field;
    if constexpr (detail::has_constant_sticking<particle_type>::value) {
      cfg.sticking = (float)particle_type::rtg_sticking;
    } else {
      field = sticking_per_disc();
    }
    rtg_context* raw = nullptr;
    check(rtg_create(&raw, cuda_device), nullptr, "no usable CUDA device");
    std::unique_ptr<rtg_context, int (*)(rtg_context*)> ctx(raw, rtg_destroy);
    check(rtg_upload_discs(raw, &points[0][0], &normals[0][0], spacing.data(), (int64_t)n), raw, "upload");
    check(rtg_set_config(raw, &cfg), raw, "configuration");
    if (window >= 0) check(rtg_set_deposit_mode(raw, RTG_DEPOSIT_WINDOW, (float)window), raw, "deposit mode");
    if (!field.empty()) check(rtg_set_sticking_field(raw, field.data(), (int64_t)n), raw, "sticking");
    check(rtg_trace(raw, (uint64_t)numofrays, seed, nullptr), raw, "trace");
    mcestimates.assign(n, 0.0f);
    std::vector<uint64_t> cnt(n, 0);
    values.assign(n, 0.0);
    relerr.assign(n, 0.0);
    vov.assign(n, 0.0);
    check(rtg_get_mc_estimates(raw, mcestimates.data()), raw, "estimates");
    check(rtg_get_hit_counts(raw, cnt.data()), raw, "hit counts");
    check(rtg_get_accumulators(raw, values.data(), nullptr, nullptr, nullptr), raw, "values");
    check(rtg_get_relative_error(raw, relerr.data()), raw, "relative error");
    check(rtg_get_vov(raw, vov.data()), raw, "variance of variance");
    hitcnts.assign(cnt.begin(), cnt.end());
  }

  std::vector<numeric_type> get_mc_estimates() { return mcestimates; }
  std::vector<size_t> get_hit_cnts() { return hitcnts; }
  // Beyond rti's device (its hit accumulator's getters, hit_accumulator.hpp:
  // 140-249): the raw flux S1 per disc in FP64, its relative error and VOV.
  std::vector<double> get_values() { return values; }
  std::vector<double> get_relative_error() { return relerr; }
  std::vector<double> get_vov() { return vov; }

 private:
  struct disc_geometry : geo::meta_geometry<numeric_type> {
    const std::vector<util::triple<numeric_type>>* nrm = nullptr;
    util::triple<numeric_type> get_normal(unsigned int id) override { return (*nrm)[id]; }
  };

  static void check(int rc, rtg_context* ctx, const char* what) {
    if (rc != RTG_OK)
      throw std::runtime_error(std::string("rti::device: ") + what + ": " + (ctx ? rtg_last_error(ctx) : "") +
                               " (rtg status " + std::to_string(rc) + ")");
  }

  std::vector<float> sticking_per_disc() {
    if constexpr (detail::has_sticking_field<particle_type>::value) {
      particle_type particle{};
      const auto f = particle.get_sticking_field();
      if (f.size() != points.size())
        throw std::runtime_error("rti::device: get_sticking_field() needs one value per disc");
      return std::vector<float>(f.begin(), f.end());
    }
    disc_geometry geo;
    geo.nrm = &normals;
    rng::splitmix_rng rng;
    rng::splitmix_rng::state st;
    particle_type particle{};
    std::vector<float> s(points.size());
    for (size_t i = 0; i < points.size(); ++i) {
      const auto& p = points[i];
      const auto& q = normals[i];
      RTCRay ray{};
      ray.org_x = p[0] + q[0];
      ray.org_y = p[1] + q[1];
      ray.org_z = p[2] + q[2];
      ray.dir_x = -q[0];
      ray.dir_y = -q[1];
      ray.dir_z = -q[2];
      ray.tnear = 1e-4f;
      ray.tfar = 1.0f;
      RTCHit hit{};
      hit.Ng_x = q[0];
      hit.Ng_y = q[1];
      hit.Ng_z = q[2];
      hit.primID = (unsigned int)i;
      hit.geomID = 1;
      particle.init_new();
      s[i] = (float)particle.get_sticking_probability(ray, hit, geo, rng, st);
    }
    return s;
  }

  std::vector<util::triple<numeric_type>> points;
  std::vector<util::triple<numeric_type>> normals;
  std::vector<numeric_type> spacing;
  std::vector<numeric_type> mcestimates;
  std::vector<size_t> hitcnts;
  std::vector<double> values, relerr, vov;
  size_t numofrays = 1024;
  bound_condition xCond = bound_condition::REFLECTIVE;
  bound_condition yCond = bound_condition::REFLECTIVE;
  numeric_type exponent = 1;
  numeric_type window = -1;  // < 0: neighbour deposit
  uint64_t seed = 0;
  int cuda_device = 0;
};
}  // namespace rti
