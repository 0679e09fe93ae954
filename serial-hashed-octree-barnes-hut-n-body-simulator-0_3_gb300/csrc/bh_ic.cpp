// Synthetic initial conditions: Plummer spheres (host code, set-up time only).
//
// The reference's own generator (src/ofApp.h:134-168) is unused by its app and is not a
// standard Plummer model, so the benchmark workloads are defined by this recipe instead:
//   radius    r = a / sqrt(U^(-2/3) - 1), U ~ Uniform(0,1), resampled when r > 10 a
//   speed     v = q * sqrt(2) * (1 + (r/a)^2)^(-1/4) * sqrt(M/a), q drawn by rejection from
//             g(q) = q^2 (1 - q^2)^(7/2) (envelope 0.1 >= max g = 0.0921)
//   directions isotropic for position and velocity; masses M/N each;
//   the sphere is shifted to its centre-of-mass frame in FP64, then the optional offsets are
//   added, and the result is rounded to FP32.
// Random numbers: xoshiro256** (Blackman & Vigna, 2018) seeded through splitmix64, uniform
// doubles from the top 53 bits. Deterministic on every platform for a given seed.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "bhgpu.h"

namespace {

struct Rng {
  uint64_t s[4];
  static uint64_t splitmix(uint64_t& x) {
    uint64_t z = (x += 0x9e3779b97f4a7c15ull);
    z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
    z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
    return z ^ (z >> 31);
  }
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (auto& w : s) w = splitmix(x);
  }
  static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
  uint64_t next() {
    uint64_t r = rotl(s[1] * 5, 7) * 9;
    uint64_t t = s[1] << 17;
    s[2] ^= s[0];
    s[3] ^= s[1];
    s[1] ^= s[2];
    s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  double uniform() { return (double)(next() >> 11) * 0x1.0p-53; }
  void direction(double out[3]) {
    double ct = 2.0 * uniform() - 1.0;
    double ph = 2.0 * M_PI * uniform();
    double st = std::sqrt(std::fmax(0.0, 1.0 - ct * ct));
    out[0] = st * std::cos(ph);
    out[1] = st * std::sin(ph);
    out[2] = ct;
  }
};

}  // namespace

extern "C" bh_status bh_plummer(uint64_t seed, size_t n, double a, double mtot, const double* pos_offset3,
                                const double* vel_offset3, float* pos_m4, float* vel4) {
  if ((n > 0 && (!pos_m4 || !vel4)) || !(a > 0) || !(mtot > 0)) return BH_ERR_INVALID_ARG;
  if (n == 0) return BH_OK;
  Rng rng(seed);
  std::vector<double> p(3 * n), v(3 * n);
  const double vscale = std::sqrt(mtot / a);
  for (size_t i = 0; i < n; ++i) {
    double r;
    for (;;) {
      double u = rng.uniform();
      if (u <= 0.0) continue;
      r = 1.0 / std::sqrt(std::pow(u, -2.0 / 3.0) - 1.0);
      if (r <= 10.0) break;
    }
    double d[3];
    rng.direction(d);
    double q;
    for (;;) {
      q = rng.uniform();
      double g = 0.1 * rng.uniform();
      if (g <= q * q * std::pow(1.0 - q * q, 3.5)) break;
    }
    double speed = q * std::sqrt(2.0) * std::pow(1.0 + r * r, -0.25) * vscale;
    double e[3];
    rng.direction(e);
    for (int k = 0; k < 3; ++k) {
      p[3 * i + k] = a * r * d[k];
      v[3 * i + k] = speed * e[k];
    }
  }
  // equal masses: the centre of mass is the plain mean
  double cp[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
  for (size_t i = 0; i < n; ++i)
    for (int k = 0; k < 3; ++k) {
      cp[k] += p[3 * i + k];
      cv[k] += v[3 * i + k];
    }
  for (int k = 0; k < 3; ++k) {
    cp[k] /= (double)n;
    cv[k] /= (double)n;
  }
  const float m = (float)(mtot / (double)n);
  for (size_t i = 0; i < n; ++i) {
    for (int k = 0; k < 3; ++k) {
      double x = p[3 * i + k] - cp[k] + (pos_offset3 ? pos_offset3[k] : 0.0);
      double u = v[3 * i + k] - cv[k] + (vel_offset3 ? vel_offset3[k] : 0.0);
      pos_m4[4 * i + k] = (float)x;
      vel4[4 * i + k] = (float)u;
    }
    pos_m4[4 * i + 3] = m;
    vel4[4 * i + 3] = 0.0f;
  }
  return BH_OK;
}
