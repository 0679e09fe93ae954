/* A plain C caller of include/bhgpu.h, written the way the reference app would bind the library
 * (the call-by-call replacement of ofApp::setup / update / draw / exit): it holds the app's own
 * 80-byte Body records, hands them to the library as they are, steps a few frames and reads them
 * back for drawing. Built and run by tests/test_c_caller.py. Exit codes: 0 frames ran, 10 no
 * usable GPU (bh_create returned BH_ERR_DEVICE), 1 any other failure. */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "bhgpu.h"

/* The reference's Body (src/Body.hpp:30-65) as the app lays it out: color at 0, displayRadius
 * at 8, position at 16, velocity at 40, mass at 64, bodyKey at 72; 80 bytes. */
typedef struct AppBody {
  unsigned char color[8];
  double displayRadius;
  double position[3];
  double velocity[3];
  double mass;
  uint64_t bodyKey;
} AppBody;

#define CHECK(call)                                                          \
  do {                                                                       \
    bh_status s_ = (call);                                                   \
    if (s_ != BH_OK) {                                                       \
      printf("%s -> %d (%s)\n", #call, (int)s_, bh_status_string(s_));       \
      return 1;                                                              \
    }                                                                        \
  } while (0)

int main(int argc, char** argv) {
  const size_t n = argc > 1 ? (size_t)strtoull(argv[1], NULL, 10) : 4444;
  const int frames = argc > 2 ? atoi(argv[2]) : 3;
  if (sizeof(AppBody) != 80) {
    printf("AppBody is %zu bytes\n", sizeof(AppBody));
    return 1;
  }
  bh_ctx* gpu = NULL;
  bh_status s = bh_create(&gpu, n, /*device=*/0);
  if (s != BH_OK) {
    printf("bh_create -> %d (%s)\n", (int)s, bh_status_string(s));
    return s == BH_ERR_DEVICE ? 10 : 1;
  }
  AppBody* bodies = (AppBody*)calloc(n, sizeof(AppBody));
  if (!bodies) return 1;
  /* ofApp::setup(): the app's scene, generated on the GPU, into the Body array */
  CHECK(bh_solar_system_device(gpu, 1, n, BH_UNITS_SI));
  CHECK(bh_get_bodies_ref(gpu, bodies, n));
  CHECK(bh_set_bodies_ref(gpu, bodies, n));
  bh_params prm;
  bh_params_default(&prm);
  prm.theta = 1.0f;                    /* src/ofApp.h:60 */
  prm.dt = 1e-3f;                      /* src/ofApp.h:62 */
  prm.eps = 0.025f;                    /* SOFTENING, src/HashedOctree.hpp:151 */
  prm.leaf_capacity = 1;
  prm.edge_factor = 1.0;
  prm.multipole = BH_MULTIPOLE_LITERAL;
  prm.acc_follows_body = 0;
  /* ofApp::update() + draw(), frame by frame */
  for (int f = 0; f < frames; ++f) {
    bh_stats st;
    memset(&st, 0, sizeof st);
    CHECK(bh_step(gpu, &prm, 1, &st));
    CHECK(bh_get_bodies_ref(gpu, bodies, n));
    if (st.error_flags != 0) {
      printf("frame %d: error flags %u\n", f, (unsigned)st.error_flags);
      return 1;
    }
  }
  for (size_t i = 0; i < n; ++i) {
    const AppBody* b = &bodies[i];
    if (!isfinite(b->position[0]) || !isfinite(b->velocity[2]) || !(b->mass > 0) || !(b->bodyKey >> 63)) {
      printf("body %zu not a valid record after the frames\n", i);
      return 1;
    }
  }
  /* ofApp::exit() */
  CHECK(bh_destroy(gpu));
  free(bodies);
  printf("ok n=%zu frames=%d\n", n, frames);
  return 0;
}
