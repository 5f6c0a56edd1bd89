/*
 * mavi_cuda.h — C ABI of libmavi_cuda.so, a GB300 (sm_103a) implementation of
 * Mavi.jl's step loop: chunk (cell-list) rebuild -> pair forces -> integration
 * -> wall handling.
 *
 * The ABI is plain C: opaque handles, plain pointers, sizes and POD parameter
 * structs. Host arrays use the reference's memory layout, so a Julia caller can
 * pass `pointer(state.pos)` of a `Vector{SVector{2,Float64}}` directly:
 * positions/velocities are interleaved [x1,y1,x2,y2,...] doubles
 * (reference: src/states.jl:75-79), rings positions are the column-major
 * (nmax x num_rings) matrix of points (src/rings/states.jl:74-81, 101).
 * Indices crossing the ABI are 0-based.
 *
 * Every entry point returns an int status (MAVI_OK == 0). Device-side failures
 * (a particle leaving the chunk grid, a chunk over capacity, a non-finite
 * position) are reported through a device error word that the library reads
 * back; kernels never trap.
 *
 * Thread-safety: one handle must be used by one host thread at a time;
 * different handles may be used concurrently (each owns its CUDA stream).
 */
#ifndef MAVI_CUDA_H
#define MAVI_CUDA_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MAVI_ABI_VERSION 1

/* ---- status codes ------------------------------------------------------ */
#define MAVI_OK                 0
#define MAVI_ERR_INVALID_ARG    1  /* bad parameter / configuration                          */
#define MAVI_ERR_CUDA           2  /* a CUDA runtime call failed (see mavi_last_error)       */
#define MAVI_ERR_OUT_OF_GRID    3  /* particle outside the chunk grid
                                      (reference raises BoundsError, src/chunks.jl:144-146) */
#define MAVI_ERR_CHUNK_OVERFLOW 4  /* more particles in a chunk than its capacity
                                      (reference raises BoundsError, src/chunks.jl:145)     */
#define MAVI_ERR_NONFINITE      5  /* NaN/Inf position                                       */
#define MAVI_ERR_OUTSIDE_SPACE  6  /* particles outside the space at construction
                                      (reference throws, src/systems.jl:76-79)              */
#define MAVI_ERR_UNSUPPORTED    7  /* combination the reference does not define             */
#define MAVI_ERR_NO_DEVICE      8  /* no CUDA device available                              */
#define MAVI_ERR_NOISE_MISSING  9  /* injected-noise mode but no noise supplied for a step  */
#define MAVI_ERR_NEIGHBOR_OVERFLOW 10 /* more rings particle neighbours than MAVI_MAX_NEIGHBORS
                                      (reference: BoundsError, src/rings/neighbors.jl:107-113) */
#define MAVI_ERR_OFFSET_RANGE   11 /* mixed form only: a particle more than 1.5 chunks from the
                                      centre of the chunk it is binned against (it moved more
                                      than a chunk within one step); its fixed-point offset
                                      would leave the exact integer range. No reference
                                      counterpart: the FP64 form has no such limit */
#define MAVI_ERR_FORCE_RANGE    12 /* mixed form, Lennard-Jones / WCA tiles only: a pair force
                                      of magnitude 2^22 or more (particles closer than ~0.37
                                      sigma), beyond the fixed-point force sums. No
                                      reference counterpart: the FP64 form has no such limit */

/* ---- enums -------------------------------------------------------------- */
/* State kinds: src/states.jl:75 (SecondLawState), :104 (SelfPropelledState),
 * src/rings/states.jl:74 (RingsState). */
#define MAVI_STATE_SECOND_LAW     0
#define MAVI_STATE_SELF_PROPELLED 1
#define MAVI_STATE_RINGS          2

/* Dynamic configs: src/configs.jl:341 (HarmTruncCfg), :380 (LenJonesCfg),
 * :399 (SzaboCfg), :410 (RunTumbleCfg), src/rings/configs.jl:326 (RingsCfg). */
#define MAVI_DYN_HARM_TRUNC 0
#define MAVI_DYN_LEN_JONES  1
#define MAVI_DYN_SZABO      2
#define MAVI_DYN_RUN_TUMBLE 3
#define MAVI_DYN_RINGS      4

/* Step functions: src/integration.jl:507 (newton_step!, velocity Verlet),
 * :517 (szabo_step!), :527 (rtp_step!), src/rings/integration.jl:522 (step!).
 * MAVI_STEP_OVERDAMPED composes reference pieces the way README.md:331-332 and
 * examples/custom_step_function.jl:43-61 tell users to write a step:
 * clean -> update_chunks! -> calc_forces! -> calc_walls_forces! ->
 * x += mobility*F*dt -> walls! -> time. */
#define MAVI_STEP_NEWTON     0
#define MAVI_STEP_SZABO      1
#define MAVI_STEP_RTP        2
#define MAVI_STEP_RINGS      3
#define MAVI_STEP_OVERDAMPED 4

/* Geometries: src/configs.jl:34 (RectangleCfg), :145 (CircleCfg), :137 (LinesCfg). */
#define MAVI_GEOM_RECTANGLE 0
#define MAVI_GEOM_CIRCLE    1
#define MAVI_GEOM_LINES     2

/* Wall types: src/configs.jl:238-244 (Rigid, Periodic, Slippery), :263 (PotentialWalls).
 * Several MaviSpace entries in one replica form ManyWalls (src/configs.jl:289-302). */
#define MAVI_WALL_RIGID     0
#define MAVI_WALL_PERIODIC  1
#define MAVI_WALL_SLIPPERY  2
#define MAVI_WALL_POTENTIAL 3

/* PotentialWalls modes: src/configs.jl:255-261. */
#define MAVI_POTMODE_OUTSIDE   0
#define MAVI_POTMODE_INSIDE    1
#define MAVI_POTMODE_REPULSION 2

/* Arithmetic of the pair loop. FP64: every operation in double (the drop-in).
 * MIXED: positions stay FP64 for update, wrap and binning; the pair loop runs in
 * FP32 instructions on exact integer chunk-centre-relative offsets (Lennard-Jones
 * and WCA terms in double-float FP32 arithmetic, compensated accumulation). */
#define MAVI_PREC_FP64  0
#define MAVI_PREC_MIXED 1

/* Noise source for Szabo / RTP / rings updates. INJECTED: the caller supplies
 * the numbers of each step (mavi_set_noise) so that two implementations can
 * consume identical noise. DEVICE: counter-based Philox4x32-10 on the GPU. */
#define MAVI_NOISE_DEVICE   0
#define MAVI_NOISE_INJECTED 1

/* Potential-energy definitions (mavi_energies). */
#define MAVI_PE_STENCIL   0  /* over the chunk-stencil pair set the forces use            */
#define MAVI_PE_ALL_PAIRS 1  /* all pairs i<j, as src/quantities.jl:46-66 does for LJ      */

#define MAVI_MAX_NEIGHBORS 15  /* neighbour list length (src/rings/rings.jl:133, 145) */
#define MAVI_MAX_SPACES 4
#define MAVI_MAX_LINES  16
#define MAVI_MAX_TYPES  4

/* ---- parameter structs -------------------------------------------------- */

/* One (wall, geometry) entry of a SpaceCfg (src/configs.jl:285-288). */
typedef struct MaviSpace {
    int32_t wall;          /* MAVI_WALL_*                                        */
    int32_t geometry;      /* MAVI_GEOM_*                                        */
    /* RectangleCfg (src/configs.jl:34-39) */
    double length, height, bl_x, bl_y;
    /* CircleCfg (src/configs.jl:145-148) */
    double radius, cx, cy;
    /* LinesCfg (src/configs.jl:137-140): segments (x1,y1,x2,y2) and optional bbox */
    int32_t num_lines;
    int32_t has_bbox;
    double lines[MAVI_MAX_LINES][4];
    double bbox_length, bbox_height, bbox_bl_x, bbox_bl_y;
    /* PotentialWalls (src/configs.jl:263-279): potential kind (MAVI_DYN_HARM_TRUNC
     * or MAVI_DYN_LEN_JONES), mode (MAVI_POTMODE_*), parameters
     * HarmTrunc: {k_rep, k_atr, dist_eq, dist_max}; LenJones: {sigma, epsilon, 0, 0} */
    int32_t pot_kind;
    int32_t pot_mode;
    double pot_params[4];
} MaviSpace;

/* Per-type rings parameters (src/rings/configs.jl:326-338) and the
 * InteractionMatrix of HarmTruncCfg (src/rings/configs.jl:257-262, 292-316).
 * k_bend is an addition (bending term, zero reproduces the reference). */
typedef struct MaviRingsCfg {
    int32_t num_types;
    int32_t num_rings;
    int32_t nmax;                           /* rows of rings_pos (max particles per ring) */
    int32_t _pad0;
    int32_t num_particles[MAVI_MAX_TYPES];  /* particles per ring of each type          */
    double p0[MAVI_MAX_TYPES];
    double relax_time[MAVI_MAX_TYPES];
    double vo[MAVI_MAX_TYPES];
    double mobility[MAVI_MAX_TYPES];
    double rot_diff[MAVI_MAX_TYPES];
    double k_area[MAVI_MAX_TYPES];
    double k_spring[MAVI_MAX_TYPES];
    double l_spring[MAVI_MAX_TYPES];
    double k_bend[MAVI_MAX_TYPES];
    double inter_k_rep[MAVI_MAX_TYPES][MAVI_MAX_TYPES];
    double inter_k_atr[MAVI_MAX_TYPES][MAVI_MAX_TYPES];
    double inter_dist_eq[MAVI_MAX_TYPES][MAVI_MAX_TYPES];
    double inter_dist_max[MAVI_MAX_TYPES][MAVI_MAX_TYPES];
} MaviRingsCfg;

/* Dynamic configuration (src/configs.jl:341-415). Fields not used by `kind`
 * are ignored. */
typedef struct MaviDynamicCfg {
    int32_t kind;          /* MAVI_DYN_*                                         */
    int32_t _pad0;
    double k_rep, k_atr, dist_eq, dist_max;                 /* HarmTruncCfg        */
    double sigma, epsilon;                                  /* LenJonesCfg / RTP   */
    double vo, mobility, relax_time, k_adh, r_eq, r_max, rot_diff; /* SzaboCfg     */
    double tumble_rate;                                     /* RunTumbleCfg        */
} MaviDynamicCfg;

/* One independent system (a Julia `System`, src/systems.jl:45-72). */
typedef struct MaviReplicaParams {
    int64_t num_particles;   /* slots: N, or nmax*num_rings for rings              */
    int32_t state_kind;      /* MAVI_STATE_*                                       */
    int32_t step_kind;       /* MAVI_STEP_*                                        */
    int32_t num_spaces;      /* 1..MAVI_MAX_SPACES; >1 means ManyWalls             */
    int32_t chunk_cols;      /* ChunksCfg.num_cols (src/configs.jl:477-480);      */
    int32_t chunk_rows;      /*   0/0 = no chunks: all-pairs forces               */
    int32_t _pad0;
    double dt;               /* IntCfg.dt (src/configs.jl:482-487)                 */
    MaviSpace spaces[MAVI_MAX_SPACES];
    MaviDynamicCfg dyn;
    MaviRingsCfg rings;
} MaviReplicaParams;

/* Options shared by all replicas of a handle. */
typedef struct MaviOptions {
    int32_t precision;       /* MAVI_PREC_*                                        */
    int32_t noise_mode;      /* MAVI_NOISE_*                                       */
    uint64_t seed;           /* Philox key for MAVI_NOISE_DEVICE                    */
    int32_t device;          /* CUDA device ordinal                                */
    int32_t use_graph;       /* capture the step in a CUDA graph when nonzero      */
    int32_t block_size;      /* threads per block for particle kernels (0 = tuned) */
    int32_t gather_mode;     /* pair gather: 0 = warp-staged shared-memory window,
                                1 = per-thread global loads chunk by chunk,
                                2 = per-thread contiguous row ranges per column
                                (0-2 add the same terms in the same order);
                                mixed Lennard-Jones / WCA with chunks only:
                                3 = Newton's third law inside tiles of chunks,
                                    one CTA per tile,
                                4 = the same tiles from a device work queue
                                    (persistent CTAs); 3 and 4 give the same
                                    bits (fixed-point sums);
                                mixed harmonic-truncated / Szabo only:
                                5 = the column gather with 2 lanes per particle,
                                6 = the same with 4 lanes (partial sums combined
                                    in a fixed order);
                                mixed Lennard-Jones only:
                                7 = the per-chunk gather with pairs at r >= 2
                                    sigma in plain FP32 and closer ones in
                                    double-float (a fixed order);
                                -1 = autotuned at creation (fastest force pass) */
} MaviOptions;

/* Work counters of the last force pass (for roofline accounting). */
typedef struct MaviStats {
    int64_t candidate_pairs;  /* chunk-stencil pairs, each unordered pair once     */
    int64_t total_particles;
    int64_t total_chunks;
    int32_t max_chunk_count;  /* largest chunk occupancy at the last rebuild        */
    int32_t gather_mode;      /* pass mode in use (MaviOptions.gather_mode 0..7)     */
} MaviStats;

/* Per-kernel device time accumulated while profiling is on (milliseconds). */
#define MAVI_KERNEL_BIN_COUNT   0  /* chunk index + histogram (fused into update)   */
#define MAVI_KERNEL_BIN_SCAN    1
#define MAVI_KERNEL_BIN_SCATTER 2
#define MAVI_KERNEL_BIN_SORT    3  /* per-chunk order + state permutation           */
#define MAVI_KERNEL_FORCE       4  /* pair-force passes (all of them)               */
#define MAVI_KERNEL_UPDATE      5  /* integration + walls (+ rings terms)           */
#define MAVI_KERNEL_OTHER       6
#define MAVI_NUM_KERNEL_KINDS   7

typedef struct MaviProfile {
    double ms[MAVI_NUM_KERNEL_KINDS];
    int64_t launches[MAVI_NUM_KERNEL_KINDS];
    int64_t steps;
    double step_ms;      /* device time from the first to the last launch of each step */
    double last_step_ms; /* the same for the most recent step                          */
} MaviProfile;

typedef struct MaviSystem MaviSystem;

/* ---- entry points ------------------------------------------------------- */

int         mavi_abi_version(void);
const char* mavi_status_string(int status);

/* Build a handle for `num_replicas` independent systems and upload their state.
 * Mirrors `System(...)` (src/systems.jl:73-114): validates that particles are
 * inside the space (check_inside, src/space_checks.jl:53-60), sizes the chunk
 * grid on the geometry's bounding box (get_chunks, src/systems.jl:14-28,
 * capacity src/chunks.jl:26-40) and runs the first update_chunks!. Rings
 * systems also run the first force evaluation (src/rings/rings.jl:280-290).
 * Host arrays are concatenated over replicas in replica order:
 *   pos, vel : 2*num_particles doubles per replica (vel NULL unless SecondLaw)
 *   pol      : num_particles (SelfPropelled) or num_rings (Rings) doubles, else NULL
 *   ring_types: num_rings int32 (1-based type ids as in the reference) or NULL */
int mavi_create(const MaviOptions* opt, int32_t num_replicas,
                const MaviReplicaParams* replicas,
                const double* pos, const double* vel, const double* pol,
                const int32_t* ring_types, MaviSystem** out);
int mavi_destroy(MaviSystem* sys);

/* Advance every replica `num_steps` steps with the replica's step function
 * (get_step_function, src/integration.jl:537-548; rings src/rings/integration.jl:545),
 * replacing `run_system(system; num_steps)` (src/run_system.jl:7-23). The steps
 * are enqueued on the handle's stream and the call returns without waiting;
 * a device error of these steps (the reference's BoundsError on a particle
 * leaving the grid or overfilling a chunk) is returned by the next call that
 * waits for results (mavi_download_state, mavi_calc_forces, mavi_get_chunks,
 * mavi_energies, mavi_update_chunks, mavi_rings_*). */
int mavi_step(MaviSystem* sys, int64_t num_steps);

/* update_chunks! for every replica (src/chunks.jl:150-161). */
int mavi_update_chunks(MaviSystem* sys);

/* Chunk contents of one replica in the reference layout
 * chunk_particles[cap, rows, cols] / num_particles_in_chunk[rows, cols]
 * (column-major, src/chunks.jl:23-24, 35-36); particle ids are 0-based and
 * ascending inside a chunk, as update_chunks! leaves them. `cap` is the
 * capacity returned by mavi_chunk_geometry. */
int mavi_chunk_geometry(MaviSystem* sys, int32_t replica, int32_t* rows,
                        int32_t* cols, int32_t* cap);
int mavi_get_chunks(MaviSystem* sys, int32_t replica, int32_t* num_in_chunk,
                    int32_t* chunk_particles);

/* One force evaluation on the current state: clean_forces! + update_chunks! +
 * calc_forces! (src/integration.jl:112-224, rings src/rings/integration.jl:197-226)
 * and, when include_walls != 0, calc_walls_forces! (src/integration.jl:228-266).
 * Writes forces of all replicas (2*N doubles, user particle order). */
int mavi_calc_forces(MaviSystem* sys, int32_t include_walls, double* forces_out);

/* Copy host state in / out (user particle order, same layout as mavi_create).
 * mavi_upload_state returns once the copy and the chunk histogram of the new
 * state are queued on the handle's stream: from page-locked host memory the
 * copy may still be in flight, so the arrays must not change before the next
 * call on this handle that waits for results (mavi_download_state,
 * mavi_calc_forces, ...); a state outside the chunk grid is reported by that
 * call. mavi_download_state waits for its copies. */
int mavi_upload_state(MaviSystem* sys, const double* pos, const double* vel,
                      const double* pol);
int mavi_download_state(MaviSystem* sys, double* pos, double* vel, double* pol);

/* mavi_download_state without the wait: the copies into pos / vel / pol are
 * queued on the handle's stream behind the steps and the call returns; the
 * arrays hold the state once mavi_synchronize (or any call that waits) has
 * returned, and must stay valid until then. From page-locked host memory the
 * copies run while the host queues work on other handles, so independent
 * replica groups on their own handles overlap one group's transfers with
 * another's steps (the reference runs independent systems of an experiment
 * batch side by side, one per thread, src/experiments.jl:271-280). No
 * reference counterpart: a transfer-scheduling call. */
int mavi_download_state_async(MaviSystem* sys, double* pos, double* vel, double* pol);

/* Waits for everything queued on the handle's stream and returns the first
 * device error of that work (as the waiting calls do), or MAVI_OK. */
int mavi_synchronize(MaviSystem* sys);

/* Noise for the next step in MAVI_NOISE_INJECTED mode: per replica, Szabo uses
 * one standard normal per particle (src/integration.jl:460), RTP two uniforms
 * per particle (src/integration.jl:493-495), rings one standard normal per ring
 * (src/rings/integration.jl:348); after all replicas' numbers, one uniform in
 * [0, 1) per random-polarisation spawn box of every replica, in replica and
 * box order (src/rings/sources.jl:24). `count` must be a positive multiple of
 * mavi_noise_count() (consecutive steps). */
int64_t mavi_noise_count(MaviSystem* sys);
int mavi_set_noise(MaviSystem* sys, const double* noise, int64_t count);
int mavi_set_seed(MaviSystem* sys, uint64_t seed);

/* Kinetic energy (src/quantities.jl:12-18) and potential energy per replica.
 * pe_mode: MAVI_PE_STENCIL or MAVI_PE_ALL_PAIRS. Outputs num_replicas doubles. */
int mavi_energies(MaviSystem* sys, int32_t pe_mode, double* ke, double* pe);

/* Energy time series on the device: num_samples times, advance every replica
 * steps_between steps (as mavi_step) and record its kinetic and potential
 * energy (as mavi_energies); everything is enqueued on the handle's stream
 * and the series is copied back once at the end. ke and pe receive
 * num_samples * num_replicas doubles, sample-major. Replaces the reference's
 * pattern of calling kinetic_energy / potential_energy (src/quantities.jl:12-66)
 * between run_system calls, without a host round trip per sample. The
 * series buffer on the device grows (one allocation) when a call needs more
 * samples than any call before it. */
int mavi_energy_series(MaviSystem* sys, int64_t num_samples, int64_t steps_between, int32_t pe_mode,
                       double* ke, double* pe);

/* Pair-distance histogram of the current state, the counts behind the pair
 * distribution g(r): counts[k] = number of unordered particle pairs of
 * `replica` (-1: all replicas summed) at distance d with floor(d / dr) == k,
 * d < r_max, dr = r_max / num_bins; d is the length of calc_diff (minimum
 * image where the reference applies it, src/integration.jl:38-52) computed
 * in FP64 without fused operations, so the counts are exact. The reference
 * has no g(r) routine; long runs of the two forms are compared by it.
 * r_max must not exceed any selected replica's chunk sides (replicas without
 * chunks: any r_max); 1 <= num_bins <= 4096. counts: num_bins uint64. */
int mavi_pair_distribution(MaviSystem* sys, int32_t replica, double r_max, int32_t num_bins,
                           uint64_t* counts);

/* time_info (src/systems.jl:30-33, src/integration.jl:500-503) of replica 0. */
int mavi_get_time(MaviSystem* sys, int64_t* num_steps, double* time);
/* Start one replica's clock at a system's time_info (a System constructed
 * with `time_info`, src/systems.jl:84-87, e.g. a loaded one); a handle
 * starts at TimeInfo(0, 0.0). Call before mavi_rings_invasions_config, whose
 * last_check is the step count at that call. The device noise counter
 * (Philox key = seed, counter = step) follows replica 0's count, so a run
 * resumed from a checkpoint with its seed continues the noise stream where it
 * stopped (as the reference's serialized RNG does) instead of replaying it. */
int mavi_set_time(MaviSystem* sys, int32_t replica, int64_t num_steps, double time);

/* Particle neighbour lists of the rings model (NeighborsCfg / ParticleNeighbors,
 * src/rings/neighbors.jl:8-136, src/rings/rings.jl:143-158): with enable != 0,
 * every pair pass of the rings step (and mavi_calc_forces) records, for each
 * particle, the candidate pairs with dist < dist_eq * tol (dist_eq of the
 * pair's types) that are in different rings, or in any ring when type_all.
 * only_count keeps the counts only. The test is the reference's FP64
 * arithmetic on FP64 positions in both precisions, so the sets are exact.
 * mavi_rings_neighbors returns, for one replica and in user slot order, the
 * counts (num_particles int32) and, unless only_count, the lists
 * (num_particles x MAVI_MAX_NEIGHBORS int32, 0-based slot ids, -1 padded; the
 * order inside a list is the GPU's visiting order, not the reference's append
 * order). Reflects the state at the last pair pass. */
int mavi_rings_neighbors_config(MaviSystem* sys, int32_t enable, int32_t only_count, int32_t type_all,
                                double tol);
int mavi_rings_neighbors(MaviSystem* sys, int32_t replica, int32_t* counts, int32_t* lists);

/* Variable number of rings (VarRingsIds, src/rings/states.jl:20-40, 152-223;
 * ActiveState, src/states.jl:14-20) with sources and sinks (SourceCfg /
 * SinkCfg, src/rings/sources.jl; RingsInfo, src/rings/rings.jl:162-186).
 *
 * mavi_rings_sources sets, for one replica, the initial active mask (one
 * int32 per ring, nonzero = active; NULL = all active) and the tuple of
 * sources and sinks in the reference's order. Every later step begins as the
 * reference's step! does (src/rings/integration.jl:522-527): the centre of
 * mass of every active ring (update_cms!), then each entry in order —
 * a sink removes every ring of the active-id view whose centre lies in its
 * geometry (process_sink!), a source finds which spawn boxes hold no particle
 * of its chunk lists (update_area_empty!, ChunksChecker / PosChecker) and
 * puts a ring into the first inactive slot for each empty box (add_ring!,
 * process_source!) — then the active ids are recomputed (update_ids!).
 * Inactive rings keep their positions and take no part in forces, update,
 * walls or chunks.
 *
 * boxes: the spawn boxes of all sources, in entry order (Source.bbox, in the
 * order of its i, j loops, src/rings/sources.jl:142-160); spawn_xy: nmax
 * points per box (Source.bbox_spawn_pos); chunk_rc: the (row, col) pairs,
 * 0-based, of every box's chunk list (ChunksChecker.ids), concatenated.
 * Random spawn polarisations (spawn_pol = :random) draw one uniform in [0, 1)
 * per random-polarisation box per step, after the rings' normals in the
 * step's noise (see mavi_noise_count); the angle is u * 2 * pi.
 * Call before the first step; the chunk lists and forces are rebuilt for the
 * active set. */
#define MAVI_SRC_SOURCE 0
#define MAVI_SRC_SINK   1
#define MAVI_SPAWN_POL_FIXED  0
#define MAVI_SPAWN_POL_RANDOM 1
#define MAVI_MAX_SOURCE_ENTRIES 8
#define MAVI_MAX_SPAWN_BOXES   64   /* per source entry */

typedef struct MaviSourceEntry {
    int32_t kind;          /* MAVI_SRC_SOURCE or MAVI_SRC_SINK                     */
    int32_t num_boxes;     /* source: spawn boxes, cfg.size[1] * cfg.size[2]        */
    int32_t pol_mode;      /* source: MAVI_SPAWN_POL_*                              */
    int32_t geometry;      /* sink: MAVI_GEOM_RECTANGLE or MAVI_GEOM_CIRCLE         */
    double pol;            /* source: fixed spawn angle                             */
    double pad;            /* source: cfg.pad (is_inside padding of the boxes)      */
    double length, height, bl_x, bl_y;   /* sink RectangleCfg                       */
    double radius, cx, cy;               /* sink CircleCfg                          */
} MaviSourceEntry;

typedef struct MaviSpawnBox {
    double bl_x, bl_y, length, height;   /* Source.bbox[i]                          */
    int32_t num_chunks;    /* chunk-list length; -1: every active particle (PosChecker) */
    int32_t _pad0;
} MaviSpawnBox;

int mavi_rings_sources(MaviSystem* sys, int32_t replica, const int32_t* active_mask, int32_t num_entries,
                       const MaviSourceEntry* entries, const MaviSpawnBox* boxes, const double* spawn_xy,
                       const int32_t* chunk_rc);
/* The rings ids of one replica: active mask (num_rings int32), uids
 * (num_rings int32, VarRingsIds.uids) and the number of active rings. */
int mavi_rings_active(MaviSystem* sys, int32_t replica, int32_t* active_mask, int32_t* uids,
                      int32_t* num_active);

/* Ring areas of one replica (num_rings doubles): RingsInfo.areas, which
 * area_forces! sets (src/rings/integration.jl:140-160) — calc_area of the
 * continuous positions of the last force evaluation, computed on demand in
 * FP64. Entries of inactive rings are computed from their parked positions. */
int mavi_rings_areas(MaviSystem* sys, int32_t replica, double* areas);

/* Invasion (src/rings/rings.jl:89-93): a particle of ring `invasor` that lies
 * inside the polygon of ring `invaded`. 1-based ring ids and the particle's
 * 1-based scalar index (to_scalar_idx, src/rings/states.jl:137-140). */
typedef struct MaviInvasion {
    int32_t invasor, invaded, p_id;
    int32_t _pad0;
} MaviInvasion;

/* Invasion detection of one replica: InvasionsCfg(steps_to_update) and the
 * ring chunks ChunksCfg(num_cols, num_rows) of RingsIntCfg
 * (src/rings/configs.jl:334-350). enable = 0 turns it off. num_cols == 0 and
 * num_rows == 0: no ring chunks (check_invasions!(system, ::Nothing),
 * src/rings/integration.jl:497-507). The call stands for the system's
 * construction: last_check becomes the replica's step count and
 * update_invasions! runs once (src/rings/rings.jl:276-284). From then on every
 * step whose num_steps - last_check >= steps_to_update runs check_invasions!
 * at the point of step! the reference does (after sources, sinks and
 * update_ids!, before the forces; src/rings/integration.jl:522-530). A step
 * that checks waits for the device once to collect the list. */
int mavi_rings_invasions_config(MaviSystem* sys, int32_t replica, int32_t enable, int64_t steps_to_update,
                                int32_t num_cols, int32_t num_rows);
/* InvasionsInfo of one replica (src/rings/rings.jl:95-100): the list in the
 * order the reference pushes it (with ring chunks the list of the last check;
 * without them every check's list appended, as the reference never empties
 * it there) and last_check. Copies min(count, capacity) entries; *count is
 * the list's length. Waits for the device. */
int mavi_rings_invasions(MaviSystem* sys, int32_t replica, MaviInvasion* out, int64_t capacity, int64_t* count,
                         int64_t* last_check);

int mavi_get_stats(MaviSystem* sys, MaviStats* stats);
/* Device-time profiling (and reset of the accumulated profile). on: 0 off,
 * 1 per kernel kind and whole step (an event pair around every launch group),
 * 2 whole step only (one event pair per step, nothing between the kernels). */
int mavi_profile_enable(MaviSystem* sys, int32_t on);
int mavi_profile_read(MaviSystem* sys, MaviProfile* prof);

/* Message of the last failure on this handle (NUL-terminated, truncated). */
int mavi_last_error(MaviSystem* sys, char* buf, int32_t len);

/* Measured FMA throughput of one GPU (FLOP/s, 2 per FMA) for
 * MAVI_PREC_FP64 (double) or MAVI_PREC_MIXED (float): the denominators of the
 * pair-force roofline. A measurement utility; the reference has no
 * counterpart. */
int mavi_fma_peak(int32_t precision, int32_t device, double* flops_per_s);

/* Chunk lists of one replica's positions that the caller already holds on the
 * current CUDA device, built WITHOUT allocating device memory. No counterpart
 * in the reference: it serves callers that cannot let a library allocate — a
 * host that owns all device memory through its own pool or budget, or one
 * that must avoid the device-wide synchronisation of cudaMalloc/cudaFree —
 * and need update_chunks! (src/chunks.jl:120-161) without a handle
 * (mavi_create allocates).
 *   params   : the replica (geometry, chunk_cols/chunk_rows, dynamic config
 *              for the particle radius and the capacity); chunks required.
 *   pos_dev  : device, 2*n doubles (interleaved x, y), 16-byte aligned.
 *   start_dev: device, rows*cols + 1 int32 written: CSR offsets over chunks
 *              in column-major order (chunk = col*rows + row), 16-byte aligned.
 *   ids_dev  : device, n int32 written: 0-based particle ids chunk by chunk,
 *              ascending inside a chunk — the reference's chunk_particles
 *              lists (mavi_get_chunks gives the same lists).
 *   stream   : cudaStream_t (NULL = legacy default stream); the call waits for
 *              it to read the status back.
 *   msg      : optional buffer (msg_len bytes) for the reason of a failure.
 * Scratch is one fixed device array inside the library: at most 1,048,576
 * chunks and a chunk capacity of at most 1024; larger requests return
 * MAVI_ERR_INVALID_ARG with the limit in msg. The first call on a device
 * loads this part of the library on that device (CUDA's lazy module loading),
 * which reserves the 4 MiB array there, and locates the array: make that
 * first call during the host's set-up. Later calls allocate nothing.
 * Every call waits for `stream` before it returns (it reads the status back).
 * A CUDA error already pending in the calling thread is returned as
 * MAVI_ERR_CUDA, named as not this call's, before anything is launched.
 * Every call clears the scratch it uses. Calls on one device share the
 * scratch, so calls that overlap in time race: serialise them per device. */
int mavi_chunk_lists_noalloc(const MaviReplicaParams* params, const double* pos_dev, int64_t n,
                             int32_t* start_dev, int32_t* ids_dev, void* stream,
                             char* msg, int32_t msg_len);

#ifdef __cplusplus
}
#endif
#endif /* MAVI_CUDA_H */
