// REF-LITERAL harness for the reference app's scene set-up and ephemeris ingest: a C ABI around
// the reference's own, unmodified SetupSolarSystem (src/PhysicsHelpers.hpp:268-683) and
// parseHorizonsFilez (src/SolarSystem.c:411-700).
//
// TEST INFRASTRUCTURE ONLY (the oracle). Only tests/ load this library, as the checker.
//
// This file contains no reference code. oracle/build_oracle.py compiles it with the reference's
// src/{MathUtils,Body}.cpp and its C utilities src/{SolarSystem,StringUtilities,FileUtilities,
// DataExtraction,GeneralUtilities,CommonDefinitions}.c, read in place from the reference
// checkout, against the headless oracle/ref_shim/ofMain.h. The output goes to oracle/_ref/.
//
// Random draws. SetupSolarSystem draws every asteroid / comet element from ofRandom, seven calls
// per body in the order e, a, inclination, node, periapsis, mean anomaly, mass. The harness
// installs a generator behind the shim's ofRandom that returns, for the k-th call, draw k % 7 of
// body 10 + k / 7 from the same counter-based uniform as the library's device generator, so the
// reference's own arithmetic runs on exactly the library's numbers.
//
// SetupSolarSystem's display-radius pass sums idx elements of a buffer holding only the large
// bodies' masses (src/PhysicsHelpers.hpp:583); the harness reserves heap room first so that
// read stays inside mapped memory (it only feeds displayRadius, which no output here uses).
#include <malloc.h>

#include <cstdint>
#include <cstdlib>
#include <vector>

#include "PhysicsHelpers.hpp"

namespace {

uint64_t g_seed = 0;
uint64_t g_calls = 0;

uint64_t mix(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

float scene_unit() {
  const uint64_t k = g_calls++;
  const uint64_t body = 10 + k / 7, draw = k % 7;
  const uint64_t z = mix(mix(g_seed + 0x9e3779b97f4a7c15ull * (body + 1)) ^ (0x632be59bd9b4e019ull * (draw + 1)));
  return (float)(((double)(z >> 11) + 0.5) * 0x1p-53);
}

}  // namespace

extern "C" {

// Runs SetupSolarSystem on n default bodies; out7[7 i ..] = position, velocity, mass (FP64).
int ref_solar_system(uint64_t seed, size_t n, double* out7) {
  mallopt(M_TRIM_THRESHOLD, 256 << 20);
  {
    std::vector<void*> room;
    for (size_t b = 0; b < 2 * n / 1024 + 64; ++b) room.push_back(std::malloc(16 << 10));
    for (void* p : room) std::free(p);
  }
  g_seed = seed;
  g_calls = 0;
  of_random_unit_hook() = &scene_unit;
  Body* bodies = new Body[n];
  SetupSolarSystem(bodies, n);
  of_random_unit_hook() = nullptr;
  for (size_t i = 0; i < n; ++i) {
    double* o = out7 + 7 * i;
    o[0] = bodies[i].position.x;
    o[1] = bodies[i].position.y;
    o[2] = bodies[i].position.z;
    o[3] = bodies[i].velocity.x;
    o[4] = bodies[i].velocity.y;
    o[5] = bodies[i].velocity.z;
    o[6] = bodies[i].mass;
  }
  delete[] bodies;
  return 0;
}

// parseHorizonsFilez on a file; out7[7 r ..] = julianDate, position, velocity. Returns the
// record count (all of them, even beyond cap).
int ref_parse_horizons(const char* path, double* out7, int cap) {
  int count = 0;
  EphemerisRecord* r = parseHorizonsFilez(path, &count);
  for (int k = 0; k < count && k < cap; ++k) {
    out7[7 * k] = r[k].julianDate;
    for (int a = 0; a < 3; ++a) {
      out7[7 * k + 1 + a] = r[k].position[a];
      out7[7 * k + 4 + a] = r[k].velocity[a];
    }
  }
  std::free(r);
  return count;
}

}  // extern "C"
