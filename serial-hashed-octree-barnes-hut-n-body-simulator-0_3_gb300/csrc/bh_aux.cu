// Around the step: initial conditions generated on the device, snapshot files, and the node
// boxes of the current tree for visualisation. None of these has a counterpart on the
// reference's hot path: the reference builds its bodies on the host
// (SetupSolarSystem / PhysicsHelpers, src/PhysicsHelpers.hpp:268-683) and draws node boxes with
// openFrameworks (visualizeTree, src/HashedOctree.cpp:939-974), which has no headless form.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "bh_internal.cuh"

namespace bh {
namespace {

constexpr int kThreads = 256;

// ---------------------------------------------------------------------------------------
// Plummer spheres on the device
// ---------------------------------------------------------------------------------------

// Counter-based uniforms: splitmix64's output mix applied to (seed, body, draw), so every body
// draws its own numbers independently of the others and of the launch shape.
__device__ __forceinline__ uint64_t mix64(uint64_t z) {
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}
__device__ __forceinline__ double uniform(uint64_t seed, uint64_t body, uint32_t draw) {
  const uint64_t z = mix64(mix64(seed + 0x9e3779b97f4a7c15ull * (body + 1)) ^ (0x632be59bd9b4e019ull * (draw + 1)));
  return ((double)(z >> 11) + 0.5) * 0x1p-53;  // in (0, 1)
}

struct Sample {
  double x[3], v[3];
};

// One body of a Plummer sphere with G = M = a = 1 (the recipe of the host generator bh_plummer):
// r = 1 / sqrt(U^(-2/3) - 1) with r > 10 rejected; speed q sqrt(2) (1 + r^2)^(-1/4) with q drawn
// by rejection from q^2 (1 - q^2)^(7/2) under the bound 0.1; isotropic directions. Each
// rejection loop has 64 rounds (the probabilities of exhausting them are below 1e-100 and
// 1e-12); an exhausted loop keeps its last draw.
__device__ Sample plummer_body(uint64_t seed, uint64_t j) {
  uint32_t draw = 0;
  double r = 0;
  for (int t = 0; t < 64; ++t) {
    const double u = uniform(seed, j, draw++);
    r = 1.0 / sqrt(pow(u, -2.0 / 3.0) - 1.0);
    if (r <= 10.0) break;
  }
  double q = 0;
  for (int t = 0; t < 64; ++t) {
    q = uniform(seed, j, draw++);
    const double g = 0.1 * uniform(seed, j, draw++);
    if (g <= q * q * pow(1.0 - q * q, 3.5)) break;
  }
  const double speed = q * sqrt(2.0) * pow(1.0 + r * r, -0.25);
  Sample s;
  double* out[2] = {s.x, s.v};
  const double mag[2] = {r, speed};
  for (int k = 0; k < 2; ++k) {
    const double ct = 2.0 * uniform(seed, j, draw++) - 1.0;
    const double ph = 6.283185307179586 * uniform(seed, j, draw++);
    const double st = sqrt(fmax(0.0, 1.0 - ct * ct));
    out[k][0] = mag[k] * st * cos(ph);
    out[k][1] = mag[k] * st * sin(ph);
    out[k][2] = mag[k] * ct;
  }
  return s;
}

// System of slot i: a binary search of the system offsets (one system when off is null).
__device__ __forceinline__ int system_of(const uint32_t* __restrict__ off, int nsys, uint32_t i) {
  if (!off) return 0;
  int lo = 0, hi = nsys - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (off[mid] <= i) lo = mid;
    else hi = mid - 1;
  }
  return lo;
}

// pass 0: per-system sums of positions and velocities (FP64; a warp whose lanes share a system
// adds once); pass 1: regenerate, subtract the system's mean, scale, write the state.
__global__ __launch_bounds__(kThreads) void k_plummer(int pass, int n, const uint32_t* __restrict__ off, int nsys,
                                                      uint64_t seed, double a, double mtot,
                                                      const double* __restrict__ offs6, double* __restrict__ sums,
                                                      float4* __restrict__ pos, float4* __restrict__ vel) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  const bool ok = i < n;
  const int s = ok ? system_of(off, nsys, (uint32_t)i) : -1;
  const uint32_t b0 = off ? off[ok ? s : 0] : 0u;
  const uint32_t nb = off ? off[(ok ? s : 0) + 1] - b0 : (uint32_t)n;
  Sample smp{};
  if (ok) smp = plummer_body(seed + (uint64_t)s, (uint64_t)i - b0);
  if (pass == 0) {
    const int lead = __shfl_sync(0xffffffffu, s, 0);
    const bool uniform_sys = __all_sync(0xffffffffu, s == lead);
    double v[6] = {smp.x[0], smp.x[1], smp.x[2], smp.v[0], smp.v[1], smp.v[2]};
    if (uniform_sys) {
#pragma unroll
      for (int k = 0; k < 6; ++k)
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_xor_sync(0xffffffffu, v[k], o);
      if ((threadIdx.x & 31) == 0 && lead >= 0)
        for (int k = 0; k < 6; ++k) atomicAdd(sums + 6 * lead + k, v[k]);
    } else if (ok) {
      for (int k = 0; k < 6; ++k) atomicAdd(sums + 6 * s + k, v[k]);
    }
    return;
  }
  if (!ok) return;
  const double inv = 1.0 / (double)nb, vs = sqrt(mtot / a);
  double x[3], u[3];
  for (int k = 0; k < 3; ++k) {
    x[k] = a * (smp.x[k] - sums[6 * s + k] * inv) + (offs6 ? offs6[k] : 0.0);
    u[k] = vs * (smp.v[k] - sums[6 * s + 3 + k] * inv) + (offs6 ? offs6[3 + k] : 0.0);
  }
  pos[i] = make_float4((float)x[0], (float)x[1], (float)x[2], (float)(mtot / (double)nb));
  vel[i] = make_float4((float)u[0], (float)u[1], (float)u[2], 0.f);
}

bh_status generate(bh_ctx* c, uint64_t seed, int n, const uint32_t* off_dev, int nsys, double a, double mtot,
                   const double* offs6_host) {
  double* sums = nullptr;
  double* offs6 = nullptr;
  BH_TRY(dalloc(&sums, (size_t)6 * nsys));
  if (offs6_host && dalloc(&offs6, 6) != BH_OK) {
    dfree(sums);
    return BH_ERR_OOM;
  }
  cudaMemsetAsync(sums, 0, sizeof(double) * 6 * nsys, c->stream);
  if (offs6) cudaMemcpyAsync(offs6, offs6_host, sizeof(double) * 6, cudaMemcpyHostToDevice, c->stream);
  const int grid = (n + kThreads - 1) / kThreads;
  c->launches += 2;
  for (int pass = 0; pass < 2; ++pass)
    k_plummer<<<grid, kThreads, 0, c->stream>>>(pass, n, off_dev, nsys, seed, a, mtot, offs6, sums, c->pos[0],
                                                 c->vel[0]);
  bh_status s = last_launch();
  if (s == BH_OK) s = cuda_status(cudaStreamSynchronize(c->stream));
  dfree(sums);
  dfree(offs6);
  return s;
}

// ---------------------------------------------------------------------------------------
// The reference's solar-system scene on the device (SetupSolarSystem,
// src/PhysicsHelpers.hpp:268-683): slot 0 the Sun, 1..8 the planets, 9 the Moon, then an
// asteroid belt up to n / 2 and an Oort cloud for the rest. One thread per body, FP64.
// ---------------------------------------------------------------------------------------

// Physical constants and the planet table of the scene (src/PhysicsHelpers.hpp:30-33,
// 298-397): the orbital elements have to be the scene's own values. The mean anomaly is given
// in degrees there but used as radians, and each planet's own mass is passed as the
// gravitational parameter; both are kept, since they decide where the planets start.
constexpr double kGrav = 6.67430e-11;
constexpr double kSunMass = 1.989e30;
constexpr double kAU = 149597870700.0;
constexpr double kDegToRad = 0.01745329252;  // the reference's toRadians factor (src/PhysicsHelpers.hpp:701-708)

struct PlanetElements {
  double e, a_au, inc_deg, node_deg, peri_deg, mean, mass;
};
__constant__ PlanetElements kPlanets[8] = {
    {0.205630, 0.387098, 7.00487, 48.331, 29.124, 174.795, 3.3011e23},         // Mercury
    {0.006772, 0.723332, 3.39471, 76.6807, 54.8523, 50.416, 4.8675e24},         // Venus
    {0.016711, 1.000000, 0.00005, 348.73936, 114.20783, 357.51716, 5.97237e24},  // Earth
    {0.093394, 1.523679, 1.85061, 49.57854, 286.502, 19.3564, 6.4171e23},       // Mars
    {0.0489, 5.2026, 1.304, 100.464, 273.867, 20.02, 1.8982e27},                // Jupiter
    {0.0565, 9.5549, 2.485, 113.665, 339.392, 317.02, 5.6834e26},               // Saturn
    {0.046381, 19.2184, 0.773, 74.006, 96.998857, 142.2386, 8.6810e25},         // Uranus
    {0.008678, 30.1104, 1.767, 131.784, 273.187, 48.12369, 1.02413e26},         // Neptune
};

// Planets and the Moon (GetCartesianFromOrbitalRadians + calculatePositionAndVelocity,
// src/PhysicsHelpers.hpp:729-811): Newton on Kepler's equation from E = M until the step is
// at most 1e-10 (100 steps at most), true anomaly, radius, then the perifocal position and the
// velocity (mu / h)(-sin nu, e + cos nu) rotated by (node, inclination, periapsis).
__device__ void kepler_true_anomaly(double e, double a, double inc, double node, double peri, double mean,
                                    double mu, double x[3], double v[3]) {
  double E = mean, step;
  int iter = 0;
  do {
    const double f = (E - e * sin(E)) - mean;
    const double fp = 1.0 - e * cos(E);
    step = -f / fp;
    E += step;
    ++iter;
  } while (fabs(step) > 1e-10 && iter < 100);
  const double nu = 2.0 * atan2(sqrt(1.0 + e) * sin(E / 2.0), sqrt(1.0 - e) * cos(E / 2.0));
  const double r = a * (1.0 - e * cos(E));
  const double cn = cos(node), sn = sin(node), cw = cos(peri), sw = sin(peri), ci = cos(inc), si = sin(inc);
  // rotation columns applied to the perifocal x and y components
  const double px = cn * cw - sn * sw * ci, qx = cn * sw + sn * cw * ci;
  const double py = sn * cw + cn * sw * ci, qy = cn * cw * ci - sn * sw;
  const double pz = sw * si, qz = cw * si;
  const double xo = r * cos(nu), yo = r * sin(nu);
  x[0] = xo * px - yo * qx;
  x[1] = xo * py + yo * qy;
  x[2] = xo * pz + yo * qz;
  const double h = sqrt(mu * a * (1.0 - e * e));
  const double vxo = -mu / h * sin(nu), vyo = mu / h * (e + cos(nu));
  v[0] = vxo * px - vyo * qx;
  v[1] = vxo * py + vyo * qy;
  v[2] = vxo * pz + vyo * qz;
}

// Asteroids and comets (computeCartesianFromOrbital, src/SolarSystem.h:33-108): 100 Newton
// steps from E = M, the perifocal position a (cos E - e, sqrt(1 - e^2) sin E) and velocity
// a Edot (-sin E, sqrt(1 - e^2) cos E) with Edot = sqrt(mu / a^3) / (1 - e cos E), rotated by
// Rz(node) Rx(inc) Rz(peri).
__device__ void kepler_eccentric(double a, double e, double inc, double node, double peri, double mean, double mu,
                                 double x[3], double v[3]) {
  double E = mean;
  for (int it = 0; it < 100; ++it) {
    const double f = (E - e * sin(E)) - mean;
    const double fp = 1.0 - e * cos(E);
    E = E - f / fp;
  }
  const double cE = cos(E), sE = sin(E), s1 = sqrt(1.0 - e * e);
  const double xp = a * (cE - e), yp = a * s1 * sE;
  const double edot = sqrt(mu / (a * a * a)) / (1.0 - e * cE);
  const double vxp = -a * edot * sE, vyp = a * edot * s1 * cE;
  const double cn = cos(node), sn = sin(node), ci = cos(inc), si = sin(inc), cw = cos(peri), sw = sin(peri);
  const double m00 = cn * cw - sn * sw * ci, m01 = -cn * sw - sn * cw * ci;
  const double m10 = sn * cw + cn * sw * ci, m11 = -sn * sw + cn * cw * ci;
  const double m20 = sw * si, m21 = cw * si;
  x[0] = m00 * xp + m01 * yp;
  x[1] = m10 * xp + m11 * yp;
  x[2] = m20 * xp + m21 * yp;
  v[0] = m00 * vxp + m01 * vyp;
  v[1] = m10 * vxp + m11 * vyp;
  v[2] = m20 * vxp + m21 * vyp;
}

// One draw of the scene's ofRandom(lo, hi) (a float): lo + (hi - lo) u in float arithmetic,
// u the body's counter-based uniform rounded to float. Rounded explicitly, so no contraction
// changes it.
__device__ __forceinline__ float scene_draw(uint64_t seed, uint64_t body, uint32_t k, float lo, float hi) {
  const float u = (float)uniform(seed, body, k);
  return __fadd_rn(lo, __fmul_rn(__fsub_rn(hi, lo), u));
}

// Body i of the scene in SI units (m, m/s, kg). Belt and cloud bodies draw, in this order,
// e, a, inclination, node, periapsis, mean anomaly (degrees) and mass from ofRandom ranges
// (src/PhysicsHelpers.hpp:492-546).
__device__ void scene_body(uint64_t seed, int i, int n, double x[3], double v[3], double* mass) {
  x[0] = x[1] = x[2] = v[0] = v[1] = v[2] = 0.0;
  if (i == 0) {
    *mass = kSunMass;
    return;
  }
  if (i <= 9) {
    const bool moon = i == 9;
    const PlanetElements& p = kPlanets[moon ? 2 : i - 1];
    kepler_true_anomaly(p.e, p.a_au * kAU, p.inc_deg * kDegToRad, p.node_deg * kDegToRad, p.peri_deg * kDegToRad,
                        p.mean, p.mass, x, v);
    *mass = p.mass;
    if (moon) {
      // Earth-centred orbit with mu = G M_earth, moved by 1.1 x Earth's position and Earth's
      // velocity (src/PhysicsHelpers.hpp:410-435)
      double xm[3], vm[3];
      kepler_true_anomaly(0.0549, 3.844e8, 5.145 * kDegToRad, 125.08 * kDegToRad, 318.15 * kDegToRad, 135.27,
                          kGrav * 5.97237e24, xm, vm);
      for (int k = 0; k < 3; ++k) {
        x[k] = xm[k] + x[k] * 1.1;
        v[k] = vm[k] + v[k];
      }
      *mass = 7.34767309e22;
    }
    return;
  }
  const bool belt = (double)i < (double)n * 0.5;
  const float e = belt ? scene_draw(seed, i, 0, 0.0f, 0.2f) : scene_draw(seed, i, 0, 0.8f, 0.99f);
  const float a = belt ? scene_draw(seed, i, 1, 2.2f, 3.2f) : scene_draw(seed, i, 1, 1000.0f, 100000.0f);
  const float inc = belt ? scene_draw(seed, i, 2, 0.0f, 15.0f) : scene_draw(seed, i, 2, 0.0f, 180.0f);
  const float node = scene_draw(seed, i, 3, 0.0f, 360.0f);
  const float peri = scene_draw(seed, i, 4, 0.0f, 360.0f);
  const float mean = scene_draw(seed, i, 5, 0.0f, 360.0f);
  const float m = belt ? scene_draw(seed, i, 6, 1e15f, 1e21f) : scene_draw(seed, i, 6, 1e12f, 1e17f);
  kepler_eccentric((double)a * kAU, (double)e, (double)inc * kDegToRad, (double)node * kDegToRad,
                   (double)peri * kDegToRad, (double)mean * kDegToRad, kGrav * kSunMass, x, v);
  *mass = (double)m;
}

// units: 0 = SI as the reference sets it up; 1 = AU, solar masses and the velocity unit of
// G = 1 (sqrt(G M_sun / AU)), where the library's G = 1 force gives the real dynamics.
__global__ __launch_bounds__(kThreads) void k_solar_system(int n, uint64_t seed, int units,
                                                           float4* __restrict__ pos, float4* __restrict__ vel) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= n) return;
  double x[3], v[3], m;
  scene_body(seed, i, n, x, v, &m);
  if (units == 1) {
    const double vu = sqrt(kGrav * kSunMass / kAU);
    for (int k = 0; k < 3; ++k) {
      x[k] /= kAU;
      v[k] /= vu;
    }
    m /= kSunMass;
  }
  pos[i] = make_float4((float)x[0], (float)x[1], (float)x[2], (float)m);
  vel[i] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.f);
}

// ---------------------------------------------------------------------------------------
// node boxes
// ---------------------------------------------------------------------------------------

// Centre and edge of every node from its key: the root cube, then per level the reference's
// child-bounds recurrence (size' = size / 2, centre' = centre + (+-0.5) size', one FP64 rounding
// per axis and level, src/HashedNode.cpp:48-70).
__global__ __launch_bounds__(kThreads) void k_node_boxes(const uint64_t* __restrict__ nkey,
                                                         const int2* __restrict__ nrange, int m, double c0,
                                                         double c1, double c2, double edge,
                                                         float4* __restrict__ box, int* __restrict__ depth,
                                                         long long* __restrict__ count) {
  const int i = blockIdx.x * kThreads + threadIdx.x;
  if (i >= m) return;
  const uint64_t key = nkey[i];
  const int d = (63 - __clzll((long long)key)) / 3;
  double c[3] = {c0, c1, c2}, s = edge;
  for (int l = d - 1; l >= 0; --l) {
    const int oct = (int)((key >> (3 * l)) & 7u);
    s = __dmul_rn(s, 0.5);
    for (int a = 0; a < 3; ++a) {
      const double dir = ((oct >> (2 - a)) & 1) ? 0.5 : -0.5;
      c[a] = __dadd_rn(c[a], __dmul_rn(dir, s));
    }
  }
  if (box) box[i] = make_float4((float)c[0], (float)c[1], (float)c[2], (float)s);
  if (depth) depth[i] = d;
  if (count) count[i] = nrange[i].y;
}

// The bounded wait every device-side spin of the library uses (the sort's and the build's
// look-backs): poll a word until it is nonzero, at most `limit` times with a short sleep, then
// give up, set the timeout bit in the error word and return.
__global__ void k_wait_flag(const uint32_t* __restrict__ flag, int limit, uint32_t* __restrict__ err) {
  if (threadIdx.x != 0) return;
  for (int i = 0; i < limit; ++i) {
    if (*((volatile const uint32_t*)flag) != 0u) return;
    __nanosleep(32);
  }
  atomicOr(err, kErrTimeout);
}

// Snapshot file: a 64-byte header, then pos_m (float4 x n), vel (float4 x n), acc (float4 x n)
// and, for an ensemble, the system offsets (u32 x (nsys + 1)). Little-endian, as both host
// architectures that run the library are.
struct SnapHeader {
  char magic[8];      // "BHGPUSNP"
  uint32_t version;   // 1
  uint32_t flags;     // bit 0: ensemble
  uint64_t n;
  uint64_t nsys;
  uint64_t reserved[4];
};
static_assert(sizeof(SnapHeader) == 64, "snapshot header is 64 bytes");

}  // namespace
}  // namespace bh

using namespace bh;

extern "C" {

bh_status bh_plummer_device(bh_ctx* c, uint64_t seed, size_t n, double a, double mtot, const double* pos_offset3,
                            const double* vel_offset3) {
  if (!c || n == 0 || n > c->cap || !(a > 0) || !(mtot > 0)) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  reset_state(c, n);
  double offs[6] = {0, 0, 0, 0, 0, 0};
  for (int k = 0; k < 3; ++k) {
    if (pos_offset3) offs[k] = pos_offset3[k];
    if (vel_offset3) offs[3 + k] = vel_offset3[k];
  }
  return generate(c, seed, (int)n, nullptr, 1, a, mtot, (pos_offset3 || vel_offset3) ? offs : nullptr);
}

bh_status bh_batch_plummer_device(bh_ctx* c, uint64_t seed, const uint32_t* sys_offsets, size_t nsys, double a,
                                  double mtot) {
  BH_TRY(check_sys_offsets(c, sys_offsets, nsys));
  if (!(a > 0) || !(mtot > 0)) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  const size_t n = sys_offsets[nsys];
  reset_state(c, n);
  BH_TRY(batch_layout(c, sys_offsets, nsys));
  return generate(c, seed, (int)n, c->sys_off, (int)nsys, a, mtot, nullptr);
}

bh_status bh_solar_system_device(bh_ctx* c, uint64_t seed, size_t n, int units) {
  if (!c || n == 0 || n > c->cap || (units != BH_UNITS_SI && units != BH_UNITS_GRAVITATIONAL))
    return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  reset_state(c, n);
  c->launches += 1;
  k_solar_system<<<(int)((n + kThreads - 1) / kThreads), kThreads, 0, c->stream>>>((int)n, seed, units, c->pos[0],
                                                                                  c->vel[0]);
  BH_TRY(last_launch());
  return cuda_status(cudaStreamSynchronize(c->stream));
}

bh_status bh_tree_boxes(bh_ctx* c, size_t cap, float* center_edge4, int32_t* depth, int64_t* count) {
  if (!c) return BH_ERR_INVALID_ARG;
  if (!c->tree_valid) return BH_ERR_NO_TREE;
  cudaSetDevice(c->device);
  const size_t m = c->n ? (size_t)c->h_level_bounds[kLevels] : 0;
  if (cap < m) return BH_ERR_INVALID_ARG;
  if (m == 0) return BH_OK;
  float4* box = nullptr;
  int* dep = nullptr;
  long long* cnt = nullptr;
  bh_status s = BH_OK;
  if (center_edge4 && s == BH_OK) s = dalloc(&box, m);
  if (depth && s == BH_OK) s = dalloc(&dep, m);
  if (count && s == BH_OK) s = dalloc(&cnt, m);
  if (s == BH_OK) {
    c->launches += 1;
    k_node_boxes<<<(int)((m + kThreads - 1) / kThreads), kThreads, 0, c->stream>>>(
        c->nkey, c->nrange, (int)m, c->tree_center[0], c->tree_center[1], c->tree_center[2], c->tree_edge, box,
        dep, cnt);
    s = last_launch();
  }
  if (s == BH_OK && box) cudaMemcpyAsync(center_edge4, box, sizeof(float4) * m, cudaMemcpyDeviceToHost, c->stream);
  if (s == BH_OK && dep) cudaMemcpyAsync(depth, dep, sizeof(int) * m, cudaMemcpyDeviceToHost, c->stream);
  if (s == BH_OK && cnt) cudaMemcpyAsync(count, cnt, sizeof(long long) * m, cudaMemcpyDeviceToHost, c->stream);
  if (s == BH_OK) s = cuda_status(cudaStreamSynchronize(c->stream));
  dfree(box);
  dfree(dep);
  dfree(cnt);
  return s;
}

bh_status bh_check_bounded_wait(bh_ctx* c, int flag_set, int limit) {
  if (!c || limit < 1 || limit > (1 << 22)) return BH_ERR_INVALID_ARG;
  cudaSetDevice(c->device);
  uint32_t* flag = nullptr;
  BH_TRY(dalloc(&flag, 1));
  clear_device_flags(c);
  cudaMemsetAsync(flag, flag_set ? 0x01 : 0x00, sizeof(uint32_t), c->stream);
  c->launches += 1;
  k_wait_flag<<<1, 32, 0, c->stream>>>(flag, limit, c->err);
  uint32_t e = 0;
  bh_status s = last_launch();
  if (s == BH_OK) s = sync_and_check(c, &e);
  dfree(flag);
  BH_TRY(s);
  clear_device_flags(c);  // the context stays usable
  return e ? err_to_status(e) : BH_OK;
}

bh_status bh_save_snapshot(bh_ctx* c, const char* path) {
  if (!c || !path) return BH_ERR_INVALID_ARG;
  const size_t n = c->n;
  std::vector<float> p(4 * n), v(4 * n), acc(4 * n);
  BH_TRY(bh_get_bodies(c, p.data(), v.data(), acc.data()));
  std::vector<uint32_t> off;
  if (c->batch) {
    off.resize((size_t)c->nsys + 1);
    cudaMemcpy(off.data(), c->sys_off, sizeof(uint32_t) * off.size(), cudaMemcpyDeviceToHost);
    BH_TRY(last_launch());
  }
  SnapHeader h{};
  std::memcpy(h.magic, "BHGPUSNP", 8);
  h.version = 1;
  h.flags = c->batch ? 1u : 0u;
  h.n = n;
  h.nsys = c->batch ? (uint64_t)c->nsys : 0;
  FILE* f = std::fopen(path, "wb");
  if (!f) return BH_ERR_INVALID_ARG;
  bool ok = std::fwrite(&h, sizeof(h), 1, f) == 1;
  if (n) {
    ok = ok && std::fwrite(p.data(), sizeof(float), p.size(), f) == p.size();
    ok = ok && std::fwrite(v.data(), sizeof(float), v.size(), f) == v.size();
    ok = ok && std::fwrite(acc.data(), sizeof(float), acc.size(), f) == acc.size();
  }
  if (!off.empty()) ok = ok && std::fwrite(off.data(), sizeof(uint32_t), off.size(), f) == off.size();
  ok = (std::fclose(f) == 0) && ok;
  return ok ? BH_OK : BH_ERR_INVALID_ARG;
}

bh_status bh_load_snapshot(bh_ctx* c, const char* path) {
  if (!c || !path) return BH_ERR_INVALID_ARG;
  FILE* f = std::fopen(path, "rb");
  if (!f) return BH_ERR_INVALID_ARG;
  SnapHeader h{};
  bool ok = std::fread(&h, sizeof(h), 1, f) == 1 && std::memcmp(h.magic, "BHGPUSNP", 8) == 0 && h.version == 1 &&
            h.n <= c->cap && (!(h.flags & 1u) || (h.nsys >= 1 && h.nsys <= 65535));
  std::vector<float> p, v, acc;
  std::vector<uint32_t> off;
  if (ok) {
    p.resize(4 * h.n);
    v.resize(4 * h.n);
    acc.resize(4 * h.n);
    ok = std::fread(p.data(), sizeof(float), p.size(), f) == p.size() &&
         std::fread(v.data(), sizeof(float), v.size(), f) == v.size() &&
         std::fread(acc.data(), sizeof(float), acc.size(), f) == acc.size();
  }
  if (ok && (h.flags & 1u)) {
    off.resize(h.nsys + 1);
    ok = std::fread(off.data(), sizeof(uint32_t), off.size(), f) == off.size() && off[h.nsys] == h.n;
  }
  std::fclose(f);
  if (!ok) return BH_ERR_INVALID_ARG;
  if (h.flags & 1u) BH_TRY(check_sys_offsets(c, off.data(), h.nsys));
  BH_TRY(bh_set_state(c, p.data(), v.data(), acc.data(), h.n));
  if (h.flags & 1u) return batch_layout(c, off.data(), h.nsys);
  return BH_OK;
}

}  // extern "C"
