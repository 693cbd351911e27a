/*
 * cgl.h — C ABI of the GB300 force-layout engine (headless cosmos.gl simulation).
 *
 * The engine replaces the per-tick force simulation behind cosmos.gl's `Graph`
 * simulation surface.  Each entry point below names the reference interface it
 * replaces (cosmos.gl `@cosmos.gl/graph` v3.4.1, paths relative to the project
 * root).  The reference has no native FFI: its host is TypeScript calling
 * luma.gl/WebGL2.  The binding a maintainer adds on the reference side is an
 * N-API addon that forwards `Graph` methods to these functions.
 *
 * Conventions
 *  - Plain pointers and sizes only.  Input arrays are COPIED at the call
 *    (the reference stores them by reference and reads them at `render()`;
 *    the data still takes effect only at `cgl_render`, as in the reference).
 *  - Output buffers are caller-allocated host memory.
 *  - Every call returns a cgl_status.  The reference never throws from these
 *    methods; non-OK statuses here correspond to its console warnings/no-ops
 *    (see cgl_last_error for the text).
 *  - One engine handle = one CUDA stream on one device.  A handle is not
 *    thread-safe; different handles are independent.
 */
#ifndef CGL_H
#define CGL_H

#include <stdint.h>
#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

#define CGL_ABI_VERSION 2u

typedef enum cgl_status {
  CGL_OK = 0,
  CGL_INVALID_ARG = 1,     /* bad argument; the call had no effect */
  CGL_OOM = 2,             /* device allocation refused (HBM budget or cudaMalloc) */
  CGL_CUDA_ERROR = 3,      /* a CUDA runtime call failed; text in cgl_last_error */
  CGL_DEVICE_TIMEOUT = 4,  /* a bounded device-side wait gave up (status word set) */
  CGL_DESTROYED = 5,       /* handle already destroyed (reference: silent no-op) */
  CGL_WARNING = 6          /* call applied with an adjustment (odd length truncated, ...) */
} cgl_status;

/* Bits of cgl_config.stage_mask: which forces a tick runs (all by default).
 * Used by stage-level parity tests; the reference always runs every enabled force. */
enum {
  CGL_STAGE_GRAVITY = 1u << 0,
  CGL_STAGE_CENTER = 1u << 1,
  CGL_STAGE_MANYBODY = 1u << 2,
  CGL_STAGE_LINK_IN = 1u << 3,
  CGL_STAGE_LINK_OUT = 1u << 4,
  CGL_STAGE_COLLISION = 1u << 5,
  CGL_STAGE_CLUSTERS = 1u << 6,
  CGL_STAGE_ALL = 0x7Fu
};

/* cgl_config.random_stream: where the random draws come from.  Both give the
 * reference's draw order and count (the jitter, one draw per link entry
 * incoming then outgoing, one peel seed per tick). */
enum {
  CGL_RANDOM_REFERENCE = 0, /* the reference's stream: random@4.1.0 float(min, max) over
                               seedrandom@3.0.5 seeded with String(randomSeed) (default) */
  CGL_RANDOM_COUNTER = 1    /* SplitMix64 by draw index: other values, but large graphs draw on the GPU */
};

/* Simulation configuration.  Field meanings and defaults follow the reference:
 * src/config.ts:56 (spaceSize), :369-456 (simulation*), :771 (randomSeed);
 * defaults src/variables.ts:10,15,19,69-82,147-148.  Fill with
 * cgl_config_defaults() and override.  "undefined" in the reference maps to
 * NaN for simulation_collision_radius and to has_random_seed = 0. */
typedef struct cgl_config {
  double space_size;                         /* spaceSize, default 4096 */
  double simulation_decay;                   /* default 5000 */
  double simulation_gravity;                 /* default 0.25 */
  double simulation_center;                  /* default 0 */
  double simulation_repulsion;               /* default 1.0 */
  double simulation_repulsion_theta;         /* default 1.15; accepted and ignored (deprecated no-op in the reference, config.ts) */
  double simulation_link_spring;             /* default 1 */
  double simulation_link_distance;           /* default 10 */
  double simulation_link_dist_random_variation_range[2]; /* default [1, 1.2] */
  double simulation_friction;                /* default 0.85 */
  double simulation_collision;               /* default 0 (off) */
  double simulation_collision_radius;        /* default NaN (= undefined: radius from point sizes) */
  double simulation_collision_padding;       /* default 0 */
  double point_default_size;                 /* default 4 (collision radius source) */
  int32_t enable_simulation;                 /* default 1 */
  int32_t has_random_seed;                   /* 0 = reference's unseeded generator (engine seeds from entropy) */
  uint64_t random_seed;                      /* randomSeed; init-only, as in the reference */
  double max_texture_dimension;              /* WebGL maxTextureDimension2D used by Store.adjustSpaceSize; 0 = no limit */
  uint32_t stage_mask;                       /* CGL_STAGE_* bits, default CGL_STAGE_ALL */
  int32_t device;                            /* CUDA device ordinal, default 0 */
  double hbm_budget_bytes;                   /* device-memory admission budget for this handle; 0 = unlimited */
  double simulation_cluster;                 /* simulationCluster, default 0.1 (config.ts:435, variables.ts:79) */
  double simulation_repulsion_from_mouse;    /* simulationRepulsionFromMouse, default 2 (variables.ts:77) */
  int32_t enable_right_click_repulsion;      /* enableRightClickRepulsion, default 0 (variables.ts:83) */
  int32_t enable_drag;                       /* enableDrag, default 0 (variables.ts:132) */
  double device_ingest_min_links;            /* the link lists (from this many links up) and, with the counter
                                                stream, the many-body jitter (from this many points up) are built
                                                on the GPU; default 65536, 0 = always, +inf = never; both builds
                                                give the same data */
  int32_t random_stream;                     /* CGL_RANDOM_REFERENCE (default) or CGL_RANDOM_COUNTER; init-only */
  int32_t rescale_positions;                 /* rescalePositions (config.ts:798): -1 undefined (default), 0 false,
                                                1 true; undefined rescales when enable_simulation is 0
                                                (Points/index.ts:396-398) */
  const char* random_seed_text;              /* with has_random_seed: randomSeed as text (UTF-8), for string seeds
                                                and non-integer numbers (the reference seeds with String(seed));
                                                NULL = random_seed in decimal.  Copied at cgl_create; init-only */
  int32_t manybody_kernel;                   /* CGL_MANYBODY_AUTO (default): the engine times its many-body
                                                kernels on a graph's first ticks and keeps the fastest; or one
                                                CGL_MANYBODY_* kernel.  Every kernel gives the same results */
} cgl_config;

typedef struct cgl_state {
  double alpha;               /* Store.alpha (FP64 on the host, as in JS) */
  double progress;            /* Graph.progress = simulationProgress */
  int32_t is_simulation_running;
  int32_t destroyed;
  uint64_t tick;              /* ticks run since create */
  uint64_t points_number;     /* applied point count (after render) */
  uint64_t links_number;      /* applied link count, including links skipped for invalid endpoints */
  uint64_t rng_draws;         /* random draws consumed so far */
} cgl_state;

typedef struct cgl_engine cgl_engine;

/* Fill *cfg with the reference's defaults (src/variables.ts). */
void cgl_config_defaults(cgl_config* cfg);

/* new Graph(div, config) — src/index.ts:167-464.  Selects the device, applies
 * Store.adjustSpaceSize (Store/index.ts:209-233) and the random seed (:452). */
cgl_status cgl_create(const cgl_config* cfg, cgl_engine** out);

/* Graph.destroy() — src/index.ts:1545.  Frees all device memory. */
cgl_status cgl_destroy(cgl_engine* e);

/* Graph.setConfig(config) — src/index.ts:500-509 (full replacement; randomSeed is
 * init-only and preserved, :1720-1724; a spaceSize change re-runs update, :1844-1851).
 * Partial updates (setConfigPartial, :519) are merged by the host shim. */
cgl_status cgl_set_config(cgl_engine* e, const cgl_config* cfg);
cgl_status cgl_get_config(cgl_engine* e, cgl_config* out);

/* Graph.setPointPositions(Float32Array) — src/index.ts:548-574.  xy = [x0,y0,x1,y1,...];
 * a NaN in either coordinate marks the point absent (helper.ts:157-159).  An odd
 * length drops the trailing value with CGL_WARNING (GraphData/index.ts:117-120).
 * At render the positions are rescaled into the space when rescale_positions is
 * 1, or when it is -1 and enable_simulation is 0 (Points.updatePositions,
 * Points/index.ts:390-413; rescaleInitialNodePositions :3134-3218).  The
 * reference rescales the caller's array in place; here the caller's array is not
 * written (cgl_get_point_positions after cgl_render returns the rescaled values). */
cgl_status cgl_set_point_positions(cgl_engine* e, const float* xy, uint64_t n_floats);
/* Graph.setPointPositions(pointPositions, dontRescale) — src/index.ts:548-553:
 * dont_rescale != 0 skips the rescale at the next render only
 * (Points.shouldSkipRescale, Points/index.ts:399-413). */
cgl_status cgl_set_point_positions_ex(cgl_engine* e, const float* xy, uint64_t n_floats, int32_t dont_rescale);

/* Graph.setLinks(Float32Array) — src/index.ts:723-734.  st = [s0,t0,s1,t1,...] of
 * point indices as floats; links with an invalid endpoint are skipped but keep
 * their index (GraphData/index.ts:534-547).  Odd length: CGL_WARNING (:296-299). */
cgl_status cgl_set_links(cgl_engine* e, const float* st, uint64_t n_floats);

/* Graph.setLinkStrength(Float32Array) — src/index.ts:836-841.  NULL/0 clears. */
cgl_status cgl_set_link_strength(cgl_engine* e, const float* strength, uint64_t n);

/* Graph.setPointSizes(Float32Array) — src/index.ts (setPointSizes); sizes feed the
 * collision radius (ForceCollision/index.ts:68-74, GraphData/index.ts:189-194). */
cgl_status cgl_set_point_sizes(cgl_engine* e, const float* sizes, uint64_t n);

/* Graph.setPinnedPoints(number[] | null) — src/index.ts:912-918; applied at once
 * (Points/index.ts:1264-1304).  Non-integer or out-of-range indices are ignored. */
cgl_status cgl_set_pinned_points(cgl_engine* e, const double* indices, uint64_t n);

/* Graph.setPointClusters((number | undefined)[]) — src/index.ts:854-859.  One
 * value per point: a non-negative integer is the point's cluster; NaN stands
 * for `undefined` (no cluster).  Negative values leave the point unclustered,
 * as in the reference (its cluster texel gets a negative row); non-integer and
 * infinite values are treated as unclustered too (the reference documents
 * integers only).  Applied at render only when n == points_number
 * (GraphData/index.ts:426-430); n = 0 or a null pointer clears the clusters. */
cgl_status cgl_set_point_clusters(cgl_engine* e, const float* clusters, uint64_t n);

/* Graph.setClusterPositions((number | undefined)[]) — src/index.ts:871-876.
 * x, y per cluster; NaN stands for `undefined` (the cluster is pulled to its
 * centre of mass, Clusters/index.ts:77-82, force-cluster.frag:41-44).  Entries
 * beyond the cluster count are ignored.  A null pointer clears them; an empty
 * non-null array counts as set (the reference runs the pass for `[]`). */
cgl_status cgl_set_cluster_positions(cgl_engine* e, const float* xy, uint64_t n_floats);

/* Graph.setPointClusterStrength(Float32Array) — src/index.ts:888-893; per-point
 * coefficient of the cluster pull (default 1), used only when n ==
 * points_number (GraphData/index.ts:436-440).  Null or n = 0 clears it. */
cgl_status cgl_set_point_cluster_strength(cgl_engine* e, const float* strength, uint64_t n);

/* Graph.render(simulationAlpha?) — src/index.ts:936-1003: ingests staged data
 * (GraphData.update :443-462, Graph.update :1987-1994, Graph.create :1635-1688).
 * alpha = NaN keeps the current alpha. */
cgl_status cgl_render(cgl_engine* e, double alpha);

/* Graph.start(alpha = 1) — src/index.ts:1457-1476. */
cgl_status cgl_start(cgl_engine* e, double alpha);
/* Graph.stop() — src/index.ts:1482-1489. */
cgl_status cgl_stop(cgl_engine* e);
/* Graph.pause() — src/index.ts:1496-1502. */
cgl_status cgl_pause(cgl_engine* e);
/* Graph.unpause() — src/index.ts:1510-1521. */
cgl_status cgl_unpause(cgl_engine* e);

/* Graph.step() × ticks — src/index.ts:1528-1540 → runSimulationStep(true)
 * (:2006-2099).  Runs even when paused.  Asynchronous on the engine stream. */
cgl_status cgl_step(cgl_engine* e, uint32_t ticks);

/* The requestAnimationFrame loop (frame() :2152-2177 → renderFrame :2237-2278):
 * while running, end the simulation when alpha < ALPHA_MIN before a tick
 * (:2164-2169, end() :2335-2339), else run a tick; at most max_ticks ticks. */
cgl_status cgl_run(cgl_engine* e, uint32_t max_ticks, uint32_t* ticks_done);

/* Interaction.  The pointer in simulation space (Store.mousePosition, which the
 * reference derives from pointer events through the zoom transform,
 * src/index.ts:updateMousePosition) and whether the right button is held
 * (Graph.isRightClickMouse).  With enable_right_click_repulsion, every frame and
 * every step first pushes the points away from the pointer (ForceMouse.run,
 * force-mouse.frag:23-38) and keeps alpha at 0.1 or more after its decay
 * (src/index.ts:2011-2016, 2082-2085). */
cgl_status cgl_set_pointer(cgl_engine* e, double x, double y, int32_t right_button_down);

/* Drag start / end (Drag/index.ts:22-36): `index` is the hovered point being
 * dragged, -1 ends the drag.  While a drag is active every frame ends by moving
 * that point to the pointer (Points.drag, drag-point.frag:22-31, called from
 * src/index.ts:2303-2310).  Ignored unless enable_drag (the reference attaches
 * no drag behaviour then); an index outside the points is INVALID_ARG. */
cgl_status cgl_set_drag(cgl_engine* e, int64_t index);

/* `frames` animation frames' simulation work (the rAF callback,
 * src/index.ts:2152-2177, and renderFrame :2237-2317), one per frame: end the
 * simulation if alpha < ALPHA_MIN while running; the right-click repulsion pass
 * if held; one tick if running; the drag pass if dragging.  *ticks_done (may be
 * null) = ticks run.  With no pointer interaction this is cgl_run plus idle
 * frames. */
cgl_status cgl_frame(cgl_engine* e, uint32_t frames, uint32_t* ticks_done);

/* Graph.getPointPositions() — src/index.ts:1106-1129; absent points read NaN.
 * out_xy holds 2 * points_number floats.  Synchronises the engine stream. */
cgl_status cgl_get_point_positions(cgl_engine* e, float* out_xy, uint64_t capacity_floats);
/* The same read-back beside the next ticks: the positions after the work
 * already queued are copied on the device (2 x 8 bytes a point on the engine
 * stream), then to out_xy (pinned host or device memory) on a copy stream
 * while the next ticks run.  It first waits for the copy the previous call
 * queued to land, so a caller alternating two buffers reads the other one
 * after each call; cgl_synchronize waits for the last.  Pageable memory:
 * CGL_INVALID_ARG (use cgl_get_point_positions). */
cgl_status cgl_enqueue_point_positions(cgl_engine* e, float* out_xy, uint64_t capacity_floats);

/* Graph.getClusterPositions() — src/index.ts:1135-1139, Clusters.getCentroidPositions
 * (Clusters/index.ts:389-423): the centre of mass of each cluster's live points,
 * x then y per cluster, sum / count in FP64 of the f32 sums (NaN for a cluster
 * with no live point).  Computed from the current positions (the reference reads
 * the texture of the pass before the last one while the simulation runs).
 * *n_out = 2 * cluster count, 0 when no per-point clusters are applied.  out may
 * be null to query the size.  Synchronises the engine stream. */
cgl_status cgl_get_cluster_positions(cgl_engine* e, double* out, uint64_t capacity_doubles, uint64_t* n_out);

/* Position hand-off to the renderer: the points texture the reference's draw
 * passes read (Points.currentPositionTexture, written by
 * buildPositionTextureData, Points/position-utils.ts:9-27): T x T RGBA32F texels,
 * T = points_texture_size, texel i = (x, y, i, 0) for i < points_number (x, y
 * NaN for absent points) and (0, 0, 0, 0) beyond.  `out` holds 4*T*T floats and
 * may be host memory (pageable or pinned) or device memory of the engine's
 * device; device and pinned host memory are written directly by one kernel (no
 * staging copy), pageable memory through a staging buffer.  Returns when the
 * texture is written. */
cgl_status cgl_get_position_texture(cgl_engine* e, float* out, uint64_t capacity_floats);
/* The same, queued on the engine stream after the work already queued and not
 * waited for: `out` must be device memory or pinned host memory; it is complete
 * after the next cgl_synchronize (or any call that synchronises).  For
 * streaming snapshots between cgl_step calls without a stall. */
cgl_status cgl_enqueue_position_texture(cgl_engine* e, float* out, uint64_t capacity_floats);

/* Graph.progress / Graph.isSimulationRunning — src/index.ts:469, :477. */
cgl_status cgl_get_state(cgl_engine* e, cgl_state* out);

/* Text of the last error or warning on this handle ("" if none). */
const char* cgl_last_error(cgl_engine* e);

/* --- Engine extensions (no counterpart in the reference) ------------------- */

/* The reference's random stream without a GPU: the first n values of
 * seedrandom(seed_text) (random@4.1.0's next(), in [0, 1)) into out.  The
 * engine seeds its stream with String(randomSeed); this lets a host or a test
 * reproduce the draws.  seed_text is UTF-8. */
cgl_status cgl_random_draws(const char* seed_text, uint64_t n, double* out);

/* The bounded wait of the one-pass cell scans, run alone on `device`: one
 * block looks back at a chunk whose status nothing ever sets, gives up after
 * its poll limit (about a second) and raises its error bit, as a scan block
 * does before the engine reports CGL_CUDA_ERROR.  *error_bits receives the
 * bits raised (CGL_ERROR_SCAN expected); the context stays usable. */
enum { CGL_ERROR_SCAN = 1 };
cgl_status cgl_check_wait_limit(int32_t device, uint32_t* error_bits);

/* Run the engine's kernels on a caller-owned cudaStream_t (NULL = engine's own). */
cgl_status cgl_set_stream(cgl_engine* e, void* cuda_stream);
/* Block until all queued work on the engine stream finished. */
cgl_status cgl_synchronize(cgl_engine* e);
/* Average device time per tick stage over `ticks` profiled ticks, in ms, via CUDA
 * events between stages (no CUDA graph).  Stage order: prepass, center, scan,
 * scatter, cells, manybody, link_in, link_out, collision_grid, collision_force,
 * clusters. */
#define CGL_NUM_STAGE_TIMES 11
cgl_status cgl_profile_stages(cgl_engine* e, uint32_t ticks, double* ms_out /*[CGL_NUM_STAGE_TIMES]*/);

/* Static layout facts of the applied data (for tests, benches and byte models). */
typedef struct cgl_layout {
  uint64_t points_number;      /* N */
  uint64_t live_points;        /* N minus absent points */
  uint64_t links_number;       /* E as given (pairs) */
  uint64_t link_entries_in;    /* valid links in the incoming CSR (== outgoing) */
  uint32_t points_texture_size;/* T = ceil(sqrt(N)) */
  uint32_t finest_grid;        /* G_f */
  uint32_t levels;             /* L */
  uint32_t max_degree_in;      /* longest link list, incoming direction */
  uint32_t max_degree_out;
  int32_t fixed_point_bits;    /* F: cell sums are exact integers in units of 2^-F */
  float fixed_point_bound;     /* |coordinate| saturates at this bound inside cell sums */
  uint32_t collision_grid;     /* collision grid size (0 until collision first runs) */
  float collision_cell_size;
  uint64_t device_bytes;       /* device memory held by the handle */
  uint32_t kernels_per_tick;   /* kernel launches one tick makes with the current data and config */
  uint32_t manybody_kernel;    /* CGL_MANYBODY_*: how the many-body pass spreads points over threads */
  uint32_t manybody_tuned;     /* 1 once manybody_kernel was chosen by timing this graph's ticks */
  uint32_t early_hubs;         /* longest incoming lists whose chains start beside the many-body pass */
  uint32_t early_points;       /* their points and link targets, whose many-body terms run first */
  uint32_t leading_out_hubs;   /* longest outgoing lists whose chains run beside the rest of their pass
                                  (from half the longest on an SM each) */
} cgl_layout;
enum {
  CGL_MANYBODY_AUTO = -1,       /* cgl_config.manybody_kernel: time the candidates, keep the fastest */
  CGL_MANYBODY_ONE_POINT = 0,   /* a thread per point */
  CGL_MANYBODY_SPLIT = 1,       /* a point's terms over 16 threads (small graphs) */
  CGL_MANYBODY_TWO_POINTS = 2   /* two points of one finest cell per thread (dense graphs) */
};
cgl_status cgl_get_layout(cgl_engine* e, cgl_layout* out);

/* Test hooks: state retained from the last tick's many-body pass. */
/* level l in [0, L): 4 floats per cell (centroid x, centroid y, count, slots), row-major. */
cgl_status cgl_debug_get_cells(cgl_engine* e, uint32_t level, float* out, uint64_t capacity_floats);
/* finest level: 8 point indices per cell in slot (hash) order, -1 = empty slot. */
cgl_status cgl_debug_get_slots(cgl_engine* e, int32_t* out, uint64_t capacity);
/* The first max_in incoming and max_out outgoing lists longer than 256 links
 * lead (cgl_layout.early_hubs, leading_out_hubs) from now on, whatever their
 * lengths (the early hubs' links still total at most an eighth of the
 * points): 0 runs every chain of that direction with the rest of its pass
 * (the incoming ones after the many-body pass), -1 restores the engine's
 * rule.  The results do not change; the hook exists to compare and time the
 * orders. */
cgl_status cgl_debug_set_leading_hubs(cgl_engine* e, int32_t max_in, int32_t max_out);

/* --- Batched engine (no counterpart in the reference) -----------------------
 * Many independent layout jobs advance together: one CUDA-graph launch per
 * tick runs every job in the batch.  Each job behaves exactly as a plain
 * engine created with the same config, given the same positions and links,
 * rendered and started at alpha 1 (cgl_create + cgl_set_point_positions +
 * cgl_set_links [+ cgl_set_point_sizes] + cgl_render + cgl_start), stepping the
 * same ticks.  Jobs join and leave between ticks (continuous batching).  Jobs
 * run gravity, center, many-body, link and collision forces; clusters and the
 * pointer's interaction need a plain engine. */
typedef struct cgl_batch cgl_batch;

typedef struct cgl_batch_info {
  uint64_t jobs;              /* jobs in the batch */
  uint64_t running_jobs;      /* jobs that still advance */
  uint64_t points;            /* points of all jobs */
  uint64_t link_entries;      /* link entries per direction, all jobs */
  uint64_t point_arena;       /* device capacities */
  uint64_t cell_arena;
  uint64_t device_bytes;
  uint32_t kernels_per_tick;
  uint32_t reserved;
} cgl_batch_info;

/* hbm_budget_bytes: device memory the batch may hold (0 = unlimited); an add
 * that would exceed it fails with CGL_OOM (admission control). */
cgl_status cgl_batch_create(int32_t device, double hbm_budget_bytes, cgl_batch** out);
cgl_status cgl_batch_destroy(cgl_batch* b);
/* Add a job; it advances on every later cgl_batch_step until it has run
 * max_ticks ticks (0 = no limit) or, when stop_below_alpha_min is set, until
 * alpha < ALPHA_MIN before a tick (the animation-frame loop's end condition,
 * src/index.ts:2164-2169). */
cgl_status cgl_batch_add(cgl_batch* b, const cgl_config* cfg, const float* xy, uint64_t n_floats, const float* links,
                         uint64_t n_link_floats, uint32_t max_ticks, int32_t stop_below_alpha_min, uint32_t* id);
/* One job of cgl_batch_add_many: cgl_batch_add's arguments, plus the job's
 * per-point sizes (Graph.setPointSizes, the collision radii; NULL = none). */
typedef struct cgl_batch_job {
  const cgl_config* cfg;
  const float* xy;
  uint64_t n_floats;
  const float* links;
  uint64_t n_link_floats;
  const float* sizes;
  uint64_t n_sizes;
  uint32_t max_ticks;
  int32_t stop_below_alpha_min;
} cgl_batch_job;
/* Add `count` jobs, each as cgl_batch_add would.  Their host work (positions,
 * the random draws of the reference's sequential stream, host link lists)
 * runs on `threads` host threads (0 = one per core) while earlier jobs upload;
 * the jobs join in order and ids[k] receives job k's id.  On a failure the
 * jobs before the failing one stay added (*added of them, may be null) and
 * its status is returned. */
cgl_status cgl_batch_add_many(cgl_batch* b, uint32_t count, const cgl_batch_job* jobs, uint32_t* ids,
                              uint32_t threads, uint32_t* added);
cgl_status cgl_batch_remove(cgl_batch* b, uint32_t id);
cgl_status cgl_batch_step(cgl_batch* b, uint32_t ticks);
cgl_status cgl_batch_synchronize(cgl_batch* b);
cgl_status cgl_batch_get_point_positions(cgl_batch* b, uint32_t id, float* out_xy, uint64_t capacity_floats);
/* The positions of `count` jobs at once: outs[k] (host memory, capacity_floats[k]
 * floats, at least 2 x points) receives job ids[k]'s [x0,y0,x1,y1,...].  One
 * device-to-host copy of the batch's point arena through a pinned staging
 * buffer kept by the batch; synchronises the batch's stream. */
cgl_status cgl_batch_get_positions_many(cgl_batch* b, uint32_t count, const uint32_t* ids, float* const* outs,
                                        const uint64_t* capacity_floats);
cgl_status cgl_batch_get_state(cgl_batch* b, uint32_t id, cgl_state* out);
cgl_status cgl_batch_get_info(cgl_batch* b, cgl_batch_info* out);
const char* cgl_batch_last_error(cgl_batch* b);

/* Many-body grid pyramid without any device allocation.  No counterpart in the
 * reference: it exists for callers that must not have a library allocate GPU
 * memory — hosts that own the whole memory budget through their own allocator,
 * code recording a CUDA graph (cudaMalloc is not allowed during capture), and
 * frame loops that cannot absorb cudaMalloc's implicit synchronisation.
 * d_xy: device positions [x0,y0,x1,y1,...] of n_points points (NaN = absent);
 * space_size: the space the engine simulates in (the configured spaceSize
 * unless max_texture_dimension reduced it, Store.adjustSpaceSize);
 * d_cells: device output, every level's cells (centroid x, centroid y, count,
 * 0), level 0 first, row-major — the cells the engine's many-body pass builds
 * for the same positions (engine levels via cgl_debug_get_cells).  Scratch is
 * a fixed 8.4 MB static device array (the largest pyramid: finest grid 512, 8
 * levels); n_points above 2^24 is rejected with CGL_INVALID_ARG.  The first
 * call on a device looks up that array's device address, so make it before any
 * stream capture; the address is kept, so after a device reset (cudaDeviceReset)
 * this entry point must not be called on that device again.  All calls share
 * the array: calls that overlap on the GPU race.  err (optional) receives the error text.  Runs on cuda_stream
 * (NULL = default stream) of the current device; calls no allocator. */
cgl_status cgl_levels_noalloc(const float* d_xy, uint64_t n_points, double space_size, float* d_cells,
                              uint64_t cells_capacity_floats, void* cuda_stream, char* err, size_t err_len);

#ifdef __cplusplus
}
#endif

#endif /* CGL_H */
