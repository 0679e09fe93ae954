/*
 * libbhgpu — GB300-native (sm_103a) per-step Barnes-Hut pipeline behind a C ABI.
 *
 * The entry points replace the per-step path of DavidRichardson02's "Serial Hashed-Octree
 * Barnes-Hut N-Body Simulator 0_3" (paths below are relative to that project's root):
 *
 *   bh_compute_bounds   OctantBounds::OctantBounds(Body*, size_t)          src/OctantUtils.cpp:27-59
 *   bh_morton_keys      computeMortonKey + interleaveBits                  src/MortonKeys.hpp:95-181
 *   bh_sort_bodies      RadixSortBodies (ThreePassRadixSortMortonKeys,
 *                       ReorderBodiesByIndexes)                            src/Body.hpp:257-302
 *   bh_build            buildLinearHashedOctreeInPlace (insertBody,
 *                       pruneEmptyNodes, computeTreeBaryCenters)           src/HashedOctree.hpp:211-244
 *   bh_node_lookup      LinearHashedOctree::lookUpNode                     src/HashedOctree.cpp:111-115
 *   bh_force            ResetVec3D + ComputeHOTOctreeForce
 *                       (TraverseHOTInteractionList,
 *                       ComputeHOTForceInteractionList, MAC)               src/HashedOctree.hpp:262-459
 *   bh_kick_drift       ComputePositionAtHalfTimeStep                      src/Body.hpp:306-313
 *   bh_kick             ComputeVelocityAndPosition                         src/Body.hpp:317-324
 *   bh_step             one frame of ofApp::update + ofApp::draw
 *                       (drawing excluded)                                 src/ofApp.cpp:169-177, 248-282
 *   bh_set_bodies_ref / bh_get_bodies_ref
 *                       the reference's 80-byte Body array (Body.hpp:30-65) <-> device state
 *
 * Conventions
 *   - Every call returns a bh_status; no exception crosses the ABI.
 *   - Host buffers belong to the caller; device buffers belong to the context and are reused
 *     across steps. A context serves one host thread at a time.
 *   - Device state is structure-of-arrays FP32: position+mass (x, y, z, m) and velocity
 *     (vx, vy, vz, 0) as float4 per body, plus accelerations (ax, ay, az, 0). Bounds and keys
 *     are computed in FP64 exactly as the reference does, so Morton keys, the sort
 *     permutation and the octree node-key set are bit-identical to the reference's on the
 *     same FP32 positions.
 *   - The body order inside a context is the order of the last bh_sort_bodies / bh_step
 *     (Morton order), as in the reference after RadixSortBodies.
 *   - All work runs on one GPU, on the context's CUDA stream (its own, or the caller's after
 *     bh_set_stream). Calls that return data to the host synchronise that stream.
 */
#ifndef BHGPU_H
#define BHGPU_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum bh_status {
  BH_OK = 0,
  BH_ERR_INVALID_ARG = 1,     /* null pointer, n above capacity, bad parameter */
  BH_ERR_OOM = 2,             /* device or pinned-host allocation failed */
  BH_ERR_DEVICE = 3,          /* a CUDA runtime call failed (no GPU, launch failure, ...) */
  BH_ERR_OVERFLOW_STACK = 4,  /* tree-walk stack overflow (device flag) */
  BH_ERR_OVERFLOW_HASH = 5,   /* node hash table probe limit reached (device flag) */
  BH_ERR_OVERFLOW_NODES = 6,  /* node arena too small; bh_step grows it and retries itself */
  BH_ERR_TIMEOUT = 7,         /* a bounded device-side wait gave up (device flag) */
  BH_ERR_NO_TREE = 8,         /* bh_force / bh_tree_* called before bh_build */
  BH_ERR_NOT_FOUND = 9,       /* bh_node_lookup: no node with that key */
  BH_ERR_OVERFLOW_TAPE = 10   /* adjoint interaction tape too small; bh_step_backward grows it itself */
} bh_status;

typedef enum bh_multipole_mode {
  /* What the reference computes today: its upsweep never runs, so every node keeps the
   * position of the first body inserted into it (insertion order = sorted order) as its
   * barycentre, the running mass sum, and a zero quadrupole (src/HashedOctree.cpp:487,597,831). */
  BH_MULTIPOLE_LITERAL = 0,
  /* The reference's intended upsweep (src/HashedOctree.cpp:721-855): centre of mass and
   * traceless quadrupole, accumulated bottom-up in FP64, used by the walk in FP32. */
  BH_MULTIPOLE_QUADRUPOLE = 1
} bh_multipole_mode;

typedef struct bh_ctx bh_ctx;

/* OctantBounds: centre = mean position; size = max_i,a (|p_ia| - c_a), the value the
 * reference uses both as the Morton half-extent and as the root node's edge. */
typedef struct bh_bounds {
  double center[3];
  double size;
} bh_bounds;

typedef struct bh_params {
  double theta;          /* opening angle of the MAC size^2 / d^2 < theta^2 */
  double eps;            /* Plummer softening (the reference hard-codes 0.025) */
  double dt;             /* time step of the kick-drift-kick leapfrog */
  int leaf_capacity;     /* bodies per leaf before it splits (the reference: 1) */
  int multipole;         /* bh_multipole_mode */
  double edge_factor;    /* root edge = edge_factor * bounds.size (the reference app: 1) */
  int acc_follows_body;  /* 1: the first half-kick uses each body's own acceleration.
                            0: the reference app's order, whose sort reorders bodies but not
                            its acceleration array (src/ofApp.cpp:176,248). */
} bh_params;

/* Per-call statistics. Stage times are CUDA-event milliseconds summed over the steps of the
 * call (filled when bh_step / bh_force get a non-null stats pointer). */
typedef struct bh_stats {
  double ms_step;          /* whole steps, first to last kernel */
  double ms_bounds;
  double ms_morton;
  double ms_sort;          /* Morton-key sort of the bodies */
  double ms_kick_drift;    /* gather into sorted order + first half-kick + drift + tree keys */
  double ms_sort_tree;     /* tree-key sort */
  double ms_build;         /* node discovery + hash table */
  double ms_upsweep;
  double ms_walk;          /* tree walk + force (+ second half-kick inside bh_step) */
  uint64_t n_nodes;
  uint64_t n_leaves;
  uint64_t interactions_cell;  /* per-body counts, summed: accepted multi-body cells */
  uint64_t interactions_p2p;   /* per-body counts, summed: single-body interactions */
  uint32_t max_depth;
  uint32_t error_flags;        /* device error word (bit set = BH_ERR_* code - 3) */
  uint32_t steps;
  uint32_t retries;            /* node-arena growths performed by bh_step */
  uint32_t kernel_launches;    /* libbhgpu kernels launched by the call */
  uint64_t walk_cell_evals;    /* cell entries the walk evaluated, 32 lane slots each */
  uint64_t walk_point_evals;   /* point entries the walk evaluated, 32 lane slots each */
} bh_stats;

typedef struct bh_node {
  uint64_t key;
  int64_t count;       /* bodies at or below the node (HOTNode::N) */
  double mass;
  double com[3];       /* barycentre used by the walk (see bh_multipole_mode) */
  double quad[6];      /* Qxx, Qxy, Qxz, Qyy, Qyz, Qzz */
  double center[3];    /* node bounds */
  double size;         /* node edge */
  int32_t depth;
  uint8_t child_byte;  /* bit o set = child in octant o exists (HOTNode::childByte) */
} bh_node;

const char* bh_status_string(bh_status s);

/* Context with room for `capacity` bodies on CUDA device `device`. */
bh_status bh_create(bh_ctx** out, size_t capacity, int device);
bh_status bh_destroy(bh_ctx* ctx);

/* Host <-> device state. pos_m4: n x (x, y, z, m); vel4: n x (vx, vy, vz, w). The physics
 * ignores w, but it travels with its body through every reordering, so a caller can keep a
 * body id there. bh_set_bodies zeroes the accelerations; bh_set_state sets them. */
bh_status bh_set_bodies(bh_ctx* ctx, const float* pos_m4, const float* vel4, size_t n);
bh_status bh_set_state(bh_ctx* ctx, const float* pos_m4, const float* vel4, const float* acc4, size_t n);
bh_status bh_get_bodies(bh_ctx* ctx, float* pos_m4, float* vel4, float* acc4);
bh_status bh_num_bodies(const bh_ctx* ctx, size_t* n);

/* The reference's Body layout (80 bytes: ofColor@0, displayRadius@8, position@16,
 * velocity@40, mass@64, bodyKey@72; FP64 vectors). Positions, velocities and masses are
 * rounded to FP32 on upload; on download the other fields are left untouched and bodyKey is
 * the last computed Morton key. */
bh_status bh_set_bodies_ref(bh_ctx* ctx, const void* bodies, size_t n);
bh_status bh_get_bodies_ref(bh_ctx* ctx, void* bodies, size_t n);

/* OctantBounds(Body*, N) of the current positions. */
bh_status bh_compute_bounds(bh_ctx* ctx, bh_bounds* out);

/* computeMortonKey(position, size) for every body; the keys stay in the context (the
 * reference stores them in Body::bodyKey) and are copied to keys_out when it is not null. */
bh_status bh_morton_keys(bh_ctx* ctx, double size, uint64_t* keys_out);

/* decodeMortonKey (src/MortonKeys.hpp:204-228) for n caller keys (host arrays: n u64 in,
 * 3n doubles out), on the context's device: each axis's 21 bits de-interleaved and mapped back
 * to x_int / 2^21 * 2 * size - size, bit for bit the reference's FP64 result. */
bh_status bh_decode_morton_keys(bh_ctx* ctx, const uint64_t* keys, size_t n, double size, double* pos3_out);

/* RadixSortBodies: stable sort of the bodies by their current keys. perm_out (optional)
 * receives, per new slot, the previous slot of the body. Like the reference, the
 * acceleration array is not reordered. */
bh_status bh_sort_bodies(bh_ctx* ctx, uint32_t* perm_out);

/* buildLinearHashedOctreeInPlace over the current bodies with the root cube
 * (center, edge): node keys by prefix truncation of the bodies' depth-21 octant paths, an
 * open-addressed device hash table over node keys, and the multipole pass of `multipole`.
 * Leaves hold up to leaf_capacity bodies; a depth-21 leaf holds any number. */
bh_status bh_build(bh_ctx* ctx, const double center[3], double edge, int leaf_capacity, int multipole);
bh_status bh_tree_size(bh_ctx* ctx, size_t* n_nodes);
/* All nodes sorted by key. Any output pointer may be null. Fails if cap < node count. */
bh_status bh_tree_nodes(bh_ctx* ctx, size_t cap, uint64_t* keys, int64_t* counts, double* mass, double* com3,
                        uint8_t* child_byte, double* quad6);
bh_status bh_node_lookup(bh_ctx* ctx, uint64_t key, bh_node* out);

/* ResetVec3D + ComputeHOTOctreeForce on the built tree: accelerations of every body,
 * written into the context and, when acc4_out is not null, copied out (n x 4 floats). */
bh_status bh_force(bh_ctx* ctx, double theta, double eps, float* acc4_out, bh_stats* stats);

/* Leapfrog halves, using the context's accelerations slot by slot. */
bh_status bh_kick_drift(bh_ctx* ctx, double dt);
bh_status bh_kick(bh_ctx* ctx, double dt);

/* nsteps frames of the reference's per-step sequence: bounds -> Morton keys -> sort ->
 * kick+drift -> build (bounds of the pre-drift positions, edge = edge_factor * size) ->
 * force -> kick. stats (optional) is filled for the call. The step runs as a captured CUDA
 * graph; with stats the graph also records an event per stage (about 5 us each, 40 us per step),
 * so callers that do not read the stage times pass NULL. A context re-captures its step graph when
 * calls switch between the two. The same holds for bh_step_host and the batched calls. */
bh_status bh_step(bh_ctx* ctx, const bh_params* params, int nsteps, bh_stats* stats);

/* One frame with the host arrays of a per-frame caller (the app's ofApp::update + draw over its
 * Body array, src/ofApp.cpp:169-282): uploads positions+mass and velocities (n x 4 floats, the
 * context's current slot order, i.e. as the previous download returned them) into the state,
 * runs one bh_step, and downloads the new positions+mass and velocities (in the new slot order).
 * The state keeps its accelerations, so a loop of calls is the same trajectory as bh_step.
 * Any pointer may be null (no copy). With page-locked buffers (bh_host_alloc or registered
 * memory) the copies overlap the step on a second stream: the velocity upload runs beside the
 * bounds, keys and sort, the position download beside the tree build and walk; a page-locked
 * velocity output that is mapped into the device's address space and 16-byte aligned is written
 * by the walk's closing kick itself (no download after the walk), any other one is downloaded
 * after the walk. The step and its copies are one CUDA graph per state parity, re-captured when
 * the buffers change. With pageable buffers the copies run before and after the step. */
bh_status bh_step_host(bh_ctx* ctx, const bh_params* params, const float* pos_m4_in, const float* vel4_in,
                       float* pos_m4_out, float* vel4_out, bh_stats* stats);

/* Batched ensembles (no counterpart in the reference, which simulates one system): nsys
 * independent systems in one context, system s owning bodies [sys_offsets[s],
 * sys_offsets[s+1]) (host array of nsys + 1 entries, sys_offsets[0] = 0, every system non-empty,
 * nsys <= 65535). bh_batch_set uploads them (like bh_set_bodies); bh_batch_step advances all
 * systems nsteps frames with bh_step's per-system semantics, in one set of launches per step
 * (captured once in a CUDA graph and replayed). Bodies never leave their system's range; within
 * it they end in the system's Morton order. bh_get_bodies downloads the whole ensemble. */
bh_status bh_batch_set(bh_ctx* ctx, const float* pos_m4, const float* vel4, const uint32_t* sys_offsets,
                       size_t nsys);
bh_status bh_batch_step(bh_ctx* ctx, const bh_params* params, int nsteps, bh_stats* stats);
/* One batched step with host arrays, as bh_step_host does for one system: uploads positions+mass
 * and velocities of all systems (n x 4 floats, the current slot order), steps, downloads them;
 * with page-locked buffers the copies overlap the step. Requires bh_batch_set first. */
bh_status bh_batch_step_host(bh_ctx* ctx, const bh_params* params, const float* pos_m4_in, const float* vel4_in,
                             float* pos_m4_out, float* vel4_out, bh_stats* stats);

/* Default parameters: theta 0.5, eps 0.025, dt 1e-3, leaf 1, quadrupole, edge 2, acc follows body. */
void bh_params_default(bh_params* p);

bh_status bh_synchronize(bh_ctx* ctx);
/* The context's CUDA stream (a cudaStream_t) and device, for callers that order their own
 * work (or bh_sort_keys_static) with the library's: every call of the context runs on it. */
bh_status bh_get_stream(bh_ctx* ctx, void** stream_out, int* device_out);
/* Runs the context's work on the caller's stream (a cudaStream_t of the context's device) from
 * now on, after finishing the work already queued; NULL returns to the context's own stream.
 * The caller keeps ownership of its stream and must not destroy it while the context uses it.
 * Step graphs are still captured on the context's own stream and launched on this one. */
bh_status bh_set_stream(bh_ctx* ctx, void* stream);

/* CUDA events on the context's stream, for timing from the caller (slots 0..63). */
bh_status bh_event_record(bh_ctx* ctx, int slot);
bh_status bh_event_elapsed_ms(bh_ctx* ctx, int slot_start, int slot_end, float* ms);
/* Writes a device buffer larger than the L2 cache on the context's stream. */
bh_status bh_flush_l2(bh_ctx* ctx);

/* Pinned host memory for fast transfers. */
bh_status bh_host_alloc(void** ptr, size_t bytes);
bh_status bh_host_free(void* ptr);

/* Measured FP32 FMA throughput of this GPU (TFLOP/s, FMA = 2 flops), from a register-only
 * kernel timed with CUDA events on the context's stream. */
bh_status bh_measure_fp32_peak(bh_ctx* ctx, double* tflops);

/* Allocation-free stable sort of (key, value) pairs in caller-owned device memory. It has no
 * counterpart in the reference. It is meant for callers that cannot call cudaMalloc where
 * they need the sort: per-frame loops and stream-callback chains, where an allocation or free
 * would synchronise the whole device, and embedders with a fixed device-memory budget. The
 * sort's scratch (ping-pong buffers, histograms, look-back words) lives in a fixed device
 * array of the library, which each GPU holds while the library is loaded, so n is limited to
 * BH_SORT_STATIC_MAX_KEYS (larger n returns BH_ERR_INVALID_ARG). Sorts stably by the full
 * 64-bit key (the same permutation as bh_sort_bodies) into keys_out / vals_out; the inputs
 * are left unchanged; asynchronous on `stream` (a cudaStream_t, NULL for the legacy default
 * stream) on the current device. status_out (optional, device memory) becomes nonzero if a
 * device-side wait gave up, in which case the output is unspecified; a give-up is reported
 * only there, so a caller that needs to know of one passes status_out.
 * The first call on each device looks up the scratch array's device address, so make it before
 * any stream capture on that device. The address is kept for the life of the process: after a
 * cudaDeviceReset (which unloads the library's device code) the entry point must not be called
 * again on that device. Every call reuses the same scratch: calls that can overlap on the GPU
 * (unordered streams, concurrent host threads) race, and the caller must order them. */
#define BH_SORT_STATIC_MAX_KEYS 65536
bh_status bh_sort_keys_static(const uint64_t* keys_in, const uint32_t* vals_in, uint64_t* keys_out,
                              uint32_t* vals_out, size_t n, void* stream, uint32_t* status_out);

/* Walk autotuner (no counterpart in the reference, whose walk is one serial loop). Times each
 * launch shape of the quadrupole tree walk (warps per block, register budget as resident blocks
 * per SM, per-warp stack depth, cell-evaluation form, and bodies per warp group: 32, or 16 / 8
 * for a single system, where more and smaller groups fill the GPU at small N; a group never
 * exceeds the 32 lanes of a warp, whose opening masks are 32-bit; ensembles walk their fixed
 * table of groups of up to 32) on the tree currently in the context: the last bh_step /
 * bh_build, or the last bh_batch_step of an ensemble. Each shape runs `trials` timed
 * force-only walks after one warm-up (the state is not changed); the fastest median becomes the
 * context's walk for quadrupole steps with eps > 0. Shapes whose stack cannot hold the tree get
 * ms = -1. */
#define BH_TUNE_MAX_VARIANTS 12
typedef struct bh_tune_result {
  int variants;
  int best;
  int warps_per_block[BH_TUNE_MAX_VARIANTS];
  int min_blocks_per_sm[BH_TUNE_MAX_VARIANTS];
  int stack_depth[BH_TUNE_MAX_VARIANTS];
  int cell_form[BH_TUNE_MAX_VARIANTS]; /* 0: three selects per cell; 1: one select on the common factor */
  int registers[BH_TUNE_MAX_VARIANTS];
  int group_size[BH_TUNE_MAX_VARIANTS]; /* bodies per warp group */
  float ms[BH_TUNE_MAX_VARIANTS];
} bh_tune_result;
bh_status bh_autotune_walk(bh_ctx* ctx, double theta, double eps, int trials, bh_tune_result* out);
/* Pins the walk's launch shape (an index of bh_tune_result, 0 = the default) without timing. */
bh_status bh_set_walk_variant(bh_ctx* ctx, int variant);

/* Conservation diagnostics of the current state (no counterpart in the reference, which reports
 * none). Kinetic energy, linear and angular momentum, mass and centre of mass are FP64 sums over
 * the bodies; the potential energy 1/2 sum m_i phi_i takes phi from the current tree (built by
 * bh_build or the last bh_step, over the current positions) with the reference's opening test at
 * theta, softening eps and the tree's multipoles (theta = 0 gives the direct sum). pot_out
 * (optional, n floats, slot order) receives phi. Returns BH_ERR_NO_TREE without a tree. */
typedef struct bh_energy {
  double kinetic;
  double potential;
  double total;
  double momentum[3];
  double angular_momentum[3];
  double mass;
  double com[3];
} bh_energy;
bh_status bh_energy_diag(bh_ctx* ctx, double theta, double eps, bh_energy* out, float* pot_out);

/* Differentiable trajectory (reverse mode). The reference has no counterpart: it only
 * integrates forward (Simulation::run, src/Simulation.cpp). bh_adjoint_forward integrates
 * nsteps kick-drift-kick steps of the quadrupole tree force from the uploaded state (bodies
 * keep their upload order, no Morton reordering; a(x_0) is computed first from a tree over
 * x_0), storing (x, v, a) every checkpoint_every steps. bh_step_backward then takes the
 * gradients of a scalar loss with respect to the final positions and velocities (float4 per
 * body, w ignored; either may be null = zero) and returns its gradients with respect to the
 * initial positions, velocities (float4, w = 0) and masses (one float per body); any output
 * may be null. The tree walks' opening decisions are held fixed (each segment is re-run from
 * its checkpoint with the walk's interaction lists recorded), so the gradient is that of the
 * piecewise-smooth map the forward pass followed. Requires multipole = quadrupole and eps > 0;
 * all host buffers are the caller's. After bh_step_backward the bodies are in the state the
 * forward pass ended in, and further backward calls with other loss gradients are allowed. */
bh_status bh_adjoint_forward(bh_ctx* ctx, const bh_params* params, int nsteps, int checkpoint_every,
                             bh_stats* stats);
bh_status bh_step_backward(bh_ctx* ctx, const float* dloss_dpos4, const float* dloss_dvel4, float* grad_pos4,
                           float* grad_vel4, float* grad_mass, bh_stats* stats);

/* Initial conditions generated on the device (no counterpart in the reference, which builds its
 * bodies on the host): a Plummer sphere by the recipe of bh_plummer (G = 1, scale radius a,
 * total mass mtot, r > 10 a rejected, centre-of-mass frame, then the optional offsets), drawn
 * with a counter-based generator per body, so the samples differ from bh_plummer's but follow
 * the same distribution; the state of the context becomes these n bodies (like bh_set_bodies).
 * bh_batch_plummer_device fills an ensemble (like bh_batch_set): system s gets the Plummer
 * sphere of seed + s with sys_offsets[s+1] - sys_offsets[s] bodies, a and mtot each. */
bh_status bh_plummer_device(bh_ctx* ctx, uint64_t seed, size_t n, double a, double mtot,
                            const double* pos_offset3, const double* vel_offset3);
bh_status bh_batch_plummer_device(bh_ctx* ctx, uint64_t seed, const uint32_t* sys_offsets, size_t nsys,
                                  double a, double mtot);

/* The reference app's own scene on the device (SetupSolarSystem, src/PhysicsHelpers.hpp:268-683;
 * computeCartesianFromOrbital, src/SolarSystem.h:33-108): body 0 the Sun at rest at the origin,
 * 1..8 Mercury..Neptune from the scene's orbital-element table (mean anomaly and gravitational
 * parameter used as the reference uses them), 9 the Moon, then asteroids (a in 2.2-3.2 AU)
 * while the index is below n / 2 and Oort-cloud comets (a in 1e3-1e5 AU) after. The random
 * elements are the reference's ofRandom ranges, drawn from a counter-based generator per body
 * (seed, body, draw) and rounded to float like ofRandom. units = BH_UNITS_SI keeps the
 * reference's metres, kilograms and m/s; BH_UNITS_GRAVITATIONAL divides by AU, the solar mass
 * and sqrt(G M_sun / AU), so the library's G = 1 force gives the scene's real dynamics (the SI
 * quadrupoles of the Oort cloud, ~m r^2 ~ 1e49, exceed the FP32 range; SI scenes need the
 * monopole-only literal mode). The state becomes these n bodies (like bh_set_bodies). */
#define BH_UNITS_SI 0
#define BH_UNITS_GRAVITATIONAL 1
bh_status bh_solar_system_device(bh_ctx* ctx, uint64_t seed, size_t n, int units);

/* Ephemeris ingest (host only): the records of a NASA JPL Horizons vector table, as
 * parseHorizonsFilez (src/SolarSystem.c:411-700; EphemerisRecord, src/SolarSystem.h) finds them
 * between the "$$SOE" and "$$EOE" lines: Julian date (TDB), X, Y, Z (km) and VX, VY, VZ (km/s).
 * Record boundaries are the reference's. By default each value is the number after its label's
 * '='; with BH_HORIZONS_LITERAL a value is read only from a token that starts with the label and
 * holds the '=' (the reference's rule, under which Horizons' "X =-1.8E+08" layout reads as 0).
 * *count receives the number of records; the first min(count, cap) go to out (which may be null
 * to count only). Returns BH_ERR_INVALID_ARG for an unreadable file and BH_ERR_NOT_FOUND when
 * the file has no $$SOE ... $$EOE region (the reference returns NULL with count 0). */
typedef struct bh_ephemeris {
  double jd_tdb;
  double pos[3];
  double vel[3];
} bh_ephemeris;
#define BH_HORIZONS_LITERAL 1
bh_status bh_parse_horizons(const char* path, int flags, bh_ephemeris* out, size_t cap, size_t* count);

/* Headless stand-in for the reference's node-box drawing (visualizeTree,
 * src/HashedOctree.cpp:939-974): for every node of the current tree (bh_build or the last
 * bh_step; node order of bh_tree_nodes) its cube as (centre x, y, z, edge), its depth and its
 * body count. Each output may be null; cap must be at least bh_tree_size. */
bh_status bh_tree_boxes(bh_ctx* ctx, size_t cap, float* center_edge4, int32_t* depth, int64_t* count);

/* Self-check of the bounded device wait (no counterpart in the reference): one thread polls a
 * device flag (set to nonzero first when flag_set, else left zero so nothing ever sets it) at
 * most `limit` times (<= 2^22, about a second) and gives up. Returns BH_OK when the flag was
 * seen, BH_ERR_TIMEOUT when the wait ran out; the context stays usable either way. */
bh_status bh_check_bounded_wait(bh_ctx* ctx, int flag_set, int limit);

/* Snapshot files (no counterpart in the reference): the bodies (slot order), their
 * accelerations (so a run continues its leapfrog exactly) and, for an ensemble, the system
 * offsets. Loading replaces the context's state like bh_set_state / bh_batch_set. */
bh_status bh_save_snapshot(bh_ctx* ctx, const char* path);
bh_status bh_load_snapshot(bh_ctx* ctx, const char* path);

/* Host-side synthetic initial conditions (set-up time, not the per-step path): a Plummer
 * sphere of n bodies, scale radius a, total mass mtot, shifted to its centre-of-mass frame,
 * then offset by pos_offset3 / vel_offset3 (either may be null). */
bh_status bh_plummer(uint64_t seed, size_t n, double a, double mtot, const double* pos_offset3,
                     const double* vel_offset3, float* pos_m4, float* vel4);

#ifdef __cplusplus
}
#endif

#endif /* BHGPU_H */
