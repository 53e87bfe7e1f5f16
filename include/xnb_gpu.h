/*
 * xnb_gpu.h -- C ABI of the GB300 (sm_103a) particle hot path.
 *
 * The library advances periodic Lennard-Jones systems with the reference's
 * per-step operator sequence (exaNBody data/config/numerical-scheme.msp:13-25):
 *   push_f_v_r ; push_f_v ; particle_displ_over ;
 *   [ move_particles ; rebuild_amr ; backup_r ; ghost_comm_scheme ;
 *     ghost_update_all ; chunk_neighbors ]  or  ghost_update_r ;
 *   zero_particle_force ; lennard_jones_force ; push_f_v
 * One "batch" holds any number of independent systems resident in HBM; every
 * entry point below that takes `sys` accepts -1 for "all systems of the batch".
 *
 * Conventions: all functions return 0 (XNB_OK) or a negative XNB_ERR_* code
 * and never throw; xnb_last_error_string() describes the last failure of the
 * calling thread. Host arrays are plain C arrays; `stream` is a cudaStream_t
 * (NULL = legacy default stream). The reference reports errors with
 * fatal_error()/abort (e.g. move_particles_across_cells.h:68-75); this ABI
 * returns codes instead so that a host runtime can recover per system.
 *
 * The reference has no C ABI: each entry point names the OperatorNode it
 * replaces (file:line inside the exaNBody tree).
 */
#ifndef XNB_GPU_H
#define XNB_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define XNB_OK 0
#define XNB_ERR_ARG (-1)      /* invalid argument or unsupported geometry */
#define XNB_ERR_CUDA (-2)     /* a CUDA runtime call failed */
#define XNB_ERR_NOMEM (-3)    /* pool or device memory exhausted */
#define XNB_ERR_CAPACITY (-4) /* neighbour list segment overflow (see xnb_system_info.error_bits) */
#define XNB_ERR_DEVICE (-5)   /* a kernel reported an error bit for a system */

/* Precision of the force traversal. */
#define XNB_PREC_FP64_EXACT 0 /* the reference functor's operations, bit-identical to its CPU path */
#define XNB_PREC_FP64 1       /* FP64, same pair set, reciprocal by Newton-Raphson, FMA */
#define XNB_PREC_MIXED 2      /* FP64 positions/displacements/accumulation/integration; FP32 r^2, r^-6, |F| */
/* Flag OR-ed into XNB_PREC_FP64 or XNB_PREC_MIXED: each pair inside rc is evaluated
 * once (lower half of the sorted list, the reference's symmetric split) and the
 * reaction is added to the partner with FP64 atomic reductions. Faster; results
 * then agree with the full-list traversal to rounding, not bit for bit, and may
 * differ in the last bits between runs. */
#define XNB_PREC_NEWTON 0x10

/* xnb_step flags */
#define XNB_STEP_HOST_SYNC 1 /* read the trigger on the host and skip the rebuild launches when idle */
#define XNB_STEP_ENERGY 2    /* also write per-particle potential energy */
/* xnb_step_persistent diagnostic: the loop's first grid barrier waits for one
 * block more than the launch has, so every wait runs out after 20 ms; the call
 * returns XNB_ERR_DEVICE and no state changes (tests the barrier's time limit) */
#define XNB_STEP_BARRIER_CHECK 0x100

/* Error bits of xnb_system_info.error_bits */
#define XNB_ERRBIT_LIST_OVERFLOW 1u
#define XNB_ERRBIT_FAR_MOVER 2u
#define XNB_ERRBIT_CELL_INDEX 4u

typedef struct xnb_batch xnb_batch;
typedef struct xnb_graph xnb_graph;

/* One periodic LJ system: domain (Domain, core/include/exanb/core/domain.h:36-129),
 * potential (LennardJonesParms, contribs/md/lennard_jones/lennard_jones.cu:40-44),
 * neighbour distances (nbh_dist, particle_neighbors/nbh_dist.cpp:45-66) and the
 * integrator step (global.dt). */
typedef struct xnb_lj_params {
  double origin[3];
  double extent[3];
  int32_t dims[3];        /* domain grid dims; >= 2 per axis */
  double cell_size;       /* >= rcut + rcut_inc (one ghost layer) */
  double rcut;            /* lennard_jones_force.rcut */
  double rcut_inc;        /* Verlet skin: nbh_dist = rcut + rcut_inc, max_displ = rcut_inc / 2 */
  double epsilon;
  double sigma;
  double dt;
  double mass;            /* used when divide_by_mass != 0 */
  int32_t divide_by_mass; /* force chain ends with divide_force_by_type_scalar: mass */
  int32_t amr_enabled;    /* rebuild_amr in-cell ordering (amr/rebuild_amr.cpp:42-61) */
  double sub_grid_density;
} xnb_lj_params;

typedef struct xnb_batch_config {
  int32_t device;
  int32_t max_systems;
  int64_t particle_capacity; /* particles over all resident systems */
  int64_t cell_capacity;     /* cells over all resident systems */
  int64_t list_capacity;     /* neighbour entries over all resident systems */
  int32_t stage_cap;         /* neighbour-build candidates staged per cell (<= 1024): cells with more go to the
                                block-per-cell build, in rounds of this size; 0 = default (640) */
  int32_t force_block;       /* threads per block of the full-list force traversal; 0 = default (64) */
} xnb_batch_config;

typedef struct xnb_system_info {
  int64_t n_particles;
  int64_t n_cells;
  int64_t list_used;  /* neighbour entries of the current lists (sum of the counts) */
  int64_t list_cap;   /* entries reserved: n_particles * per-particle slot */
  int64_t rebuilds;   /* neighbour-list rebuilds since xnb_init_particles */
  uint32_t error_bits;
  uint32_t max_cell;  /* largest cell occupancy after the last rebin */
  int32_t active;
  uint32_t max_nbr;   /* largest per-particle list count of the last build */
} xnb_system_info;

const char* xnb_last_error_string(void);
int xnb_version(void);

/* Device pools for one batch. */
int xnb_batch_create(const xnb_batch_config* cfg, xnb_batch** out);
int xnb_batch_destroy(xnb_batch* b);
/* Bytes of device memory a system of n particles and ncells cells needs, with
 * a neighbour slot of list_per_particle entries per particle (admission control). */
int64_t xnb_system_bytes(int64_t n, int64_t ncells, double list_per_particle);

/* Upload one system. cell_counts == NULL: particles are placed in the cell of
 * their periodic location, in input order (stable). Otherwise the arrays are
 * given per interior cell (linear order (k*Dj+j)*Di+i) as the reference grid
 * holds them, and positions may lie outside their cell (the reference's
 * lattice generator then relies on init's move_particles). Each particle's
 * neighbour list has a fixed slot; a host-synchronised build sizes the slot to
 * list_factor x the largest count + 16 (>= 1; 0 = 1.3), and a build without
 * host synchronisation that outgrows it flags XNB_ERRBIT_LIST_OVERFLOW. */
int xnb_system_add(xnb_batch* b, const xnb_lj_params* p, int64_t n, const double* rx, const double* ry,
                   const double* rz, const double* vx, const double* vy, const double* vz, const uint64_t* id,
                   const int64_t* cell_counts, double list_factor, void* stream, int32_t* sys_out);
int xnb_system_remove(xnb_batch* b, int32_t sys, void* stream);
int xnb_system_info_get(xnb_batch* b, int32_t sys, xnb_system_info* info, void* stream);
/* Particles in storage order (cells in linear order, then in-cell order).
 * Any output pointer may be NULL. */
int xnb_system_download(xnb_batch* b, int32_t sys, double* rx, double* ry, double* rz, double* vx, double* vy,
                        double* vz, double* fx, double* fy, double* fz, uint64_t* id, int32_t* cell, double* pe,
                        void* stream);
/* Neighbour pairs as particle ids in list order; nbh_count gets one length per
 * particle (storage order). cap is the size of id_a/id_b; n_out the pair count. */
int xnb_system_pairs(xnb_batch* b, int32_t sys, uint64_t* id_a, uint64_t* id_b, int32_t* nbh_count, int64_t cap,
                     int64_t* n_out, void* stream);
/* The same for the particles [first, first + count) of the system (storage
 * order): partner ids in list order and one length per particle of the range,
 * so that large systems cross to the host in slices. Synchronises. */
int xnb_system_pairs_range(xnb_batch* b, int32_t sys, int64_t first, int64_t count, uint64_t* id_b,
                           int32_t* nbh_count, int64_t cap, int64_t* n_out, void* stream);
/* Kinetic 0.5*m*v^2 and truncated-and-shifted LJ energy of the last force call
 * made with energies. */
int xnb_system_energy(xnb_batch* b, int32_t sys, double* ke, double* pe, void* stream);

/* ---- reference operators (sys = -1: all systems) ---- */

/* init_particles (data/config/update-particles.msp:31-36) then
 * compute_all_forces_energy (numerical-scheme.msp:8-11). */
int xnb_init_particles(xnb_batch* b, int32_t sys, int32_t precision, void* stream);
/* push_f_v_r: PushVec3SecondOrderXForm (defbox/include/exanb/defbox/push_vec3_2nd_order.h:85-117). */
int xnb_push_f_v_r(xnb_batch* b, int32_t sys, double dt_scale, void* stream);
/* push_f_v: PushVec3FirstOrder (defbox/include/exanb/defbox/push_vec3_1st_order.h:79-106). */
int xnb_push_f_v(xnb_batch* b, int32_t sys, double dt_scale, void* stream);
/* particle_displ_over: ParticleDisplacementOver (mpi/particle_displ_over.cu:93-177).
 * Synchronises the stream; count_out[sys or 0] = particles over the threshold. */
int xnb_particle_displ_over(xnb_batch* b, int32_t sys, int64_t* count_out, void* stream);
/* update_particles_full (update-particles.msp:62-68): move_particles
 * (grid_cell_particles/move_particles.cpp:39-48), migrate_cell_particles,
 * rebuild_amr, backup_r, ghost_comm_scheme, ghost_update_all, chunk_neighbors. */
int xnb_update_particles_full(xnb_batch* b, int32_t sys, void* stream);
/* chunk_neighbors: BuildChunkNeighbors (particle_neighbors/chunk_neighbors.cpp:47-72). */
int xnb_chunk_neighbors(xnb_batch* b, int32_t sys, void* stream);
/* backup_r: PositionBackupNode (io/backup_r.cpp:35-107). */
int xnb_backup_r(xnb_batch* b, int32_t sys, void* stream);
/* zero_particle_force (compute/zero_particle_force.cu:17-53) + lennard_jones_force
 * (contribs/md/lennard_jones/lennard_jones.cu:171-213) [+ divide_force_by_type_scalar]. */
int xnb_lennard_jones_force(xnb_batch* b, int32_t sys, int32_t precision, int32_t with_energy, void* stream);
/* ghost_update_r (mpi/update_ghosts.cu:58): ghost images are evaluated on the
 * fly from their owners, so there is nothing to copy; kept for the operator set. */
int xnb_ghost_update_r(xnb_batch* b, int32_t sys, void* stream);

/* ---- fused numerical scheme ---- */

/* nsteps of numerical_scheme (numerical-scheme.msp:21-25) for every system of
 * the batch, fused into three kernels per step plus the rebuild path. */
int xnb_step(xnb_batch* b, int32_t nsteps, int32_t precision, int32_t flags, void* stream);
/* The same nsteps as a persistent step loop: one cooperative launch advances
 * every system step after step (first half and trigger, a grid barrier, forces
 * with the second-half kick, a grid barrier), one thread per particle on full
 * lists, until a step's trigger fires; that step's rebuild path and forces run
 * as separate launches (host-synchronised, as XNB_STEP_HOST_SYNC), then the loop
 * resumes. States are bitwise those of xnb_step. The barriers' waits are bounded
 * (4 s): a wait that runs out ends the launch and the call returns
 * XNB_ERR_DEVICE. XNB_PREC_NEWTON is refused. Flags: XNB_STEP_ENERGY,
 * XNB_STEP_BARRIER_CHECK (XNB_STEP_HOST_SYNC is implied). Synchronises. */
int xnb_step_persistent(xnb_batch* b, int32_t nsteps, int32_t precision, int32_t flags, void* stream);
/* Captures nsteps of the fused step (device-side trigger, no host sync) as a CUDA graph. */
int xnb_step_graph_create(xnb_batch* b, int32_t nsteps, int32_t precision, int32_t flags, void* stream,
                          xnb_graph** out);
/* Launches the captured steps; XNB_ERR_ARG when the batch's extent (the
 * high-water marks of its particle and cell pools, the number of system slots)
 * or launch configuration changed since capture: systems added beyond the
 * captured extent would not be stepped, so the graph must be captured again. */
int xnb_graph_launch(xnb_graph* g, void* stream);
/* 1 when the graph still covers the batch as it is (xnb_graph_launch accepts it), else 0. */
int xnb_graph_is_current(const xnb_graph* g);
int xnb_graph_destroy(xnb_graph* g);
/* Any device error bit set on any system -> XNB_ERR_DEVICE / XNB_ERR_CAPACITY (synchronises). */
int xnb_check_errors(xnb_batch* b, void* stream);
/* Kernels this batch has enqueued so far (host-side count, for launch accounting;
 * the reference's equivalent bookkeeping lives in onika's profiling layer). */
int64_t xnb_stats_kernel_launches(const xnb_batch* b);

/* ---- tuning ---- */

typedef struct xnb_tuning {
  int32_t stage_cap;          /* neighbour-build candidates staged per cell (see xnb_batch_config) */
  int32_t force_block;        /* threads per block of the full-list force traversal */
  int32_t newton;             /* 1: XNB_PREC_NEWTON traversal */
  int32_t trials;             /* configurations timed */
  double atom_steps_per_s;    /* the chosen configuration's measured rate */
  int32_t build_form;         /* XNB_BUILD_ROWS or XNB_BUILD_WARP */
  int32_t force_lanes;        /* threads per particle of the FP64 / mixed full-list force traversal */
  int32_t force_form;         /* the batch's force form (XNB_FORCE_THREAD or XNB_FORCE_STAGED; not searched) */
  int32_t reserved;
} xnb_tuning;

/* Threads per particle (1, 2 or 4) of the FP64 and mixed full-list force
 * traversals: the particle's list is split in 8-entry blocks dealt round-robin
 * to the threads and their partial sums combined in a fixed order, so results
 * are reproducible and agree with one thread per particle to rounding.
 * FP64_EXACT always runs one thread per particle. */
int xnb_batch_set_force_lanes(xnb_batch* b, int32_t lanes);

/* Form of the mixed-precision full-list force traversal:
 * XNB_FORCE_THREAD: one thread per particle, neighbours gathered from global memory (default);
 * XNB_FORCE_STAGED: one block per segment of 8 x-adjacent cells of a row, whose
 *   neighbourhood (9 rows of 10 cells, periodic images included) is copied into
 *   shared memory first; the lists are read in a compact (cell group, index in
 *   cell) form written after each build. Forces, energies and velocities are
 *   bitwise equal to XNB_FORCE_THREAD, and slower (4.65 against 2.62 ms per
 *   4M-atom force call, plus 3 ms per rebuild for the compact entries, on
 *   GB300). Switching it on allocates 2 bytes per
 *   list entry of the batch and a segment table, and compacts the current lists
 *   (synchronises the device). FP64 and Newton traversals are unaffected. */
#define XNB_FORCE_THREAD 0
#define XNB_FORCE_STAGED 1
int xnb_batch_set_force_form(xnb_batch* b, int32_t form);

/* Neighbour-build kernels (both give the same lists, the reference's):
 * XNB_BUILD_ROWS: one warp per cell, one lane per particle (two for cells of
 *   33-64 particles); the 27 neighbour cells staged as 9 rows of three
 *   x-adjacent cells, each cell's mirrors one bulk copy (cp.async.bulk) into
 *   shared memory, the next row's copy in flight while the current row is tested.
 * XNB_BUILD_WARP: one warp per cell, one lane per candidate; the whole 27-cell
 *   block (up to stage_cap candidates) staged by the warp, six particles tested
 *   per staged load with a ballot each.
 * Cells neither form takes (more than 64 particles, or candidates over the
 * stage) are built block-per-cell. */
#define XNB_BUILD_ROWS 0
#define XNB_BUILD_WARP 1
/* XNB_BUILD_HALF: each pair of cells once (a cell and the 13 cells after it in
 *   (dk, dj, di) order, one warp per cell, lanes over the other cell's
 *   particles): one distance decision per pair sets a bit in both particles'
 *   per-cell masks (each direction with its own ghost filter and, near nbh, its
 *   own FP64 test); a second pass writes each list from its 27 masks. Selecting
 *   it allocates 27 x 8 bytes per particle of capacity. A system with a cell of
 *   more than 64 particles is built by XNB_BUILD_WARP instead. Slower than
 *   XNB_BUILD_WARP on GB300 (10.5 against 3.8 ms per 4M-atom rebuild); not
 *   searched by xnb_autotune. */
#define XNB_BUILD_HALF 2
int xnb_batch_set_build_form(xnb_batch* b, int32_t form);

/* Sub-cell pair pruning of the neighbour build (on by default), after
 * max_distance_sub_cell_pairs / AmrSubCellPairCache
 * (amr/lib/amr_grid_algorithm.cpp:102-218, used at
 * particle_neighbors/include/exanb/particle_neighbors/chunk_neighbors_execute.h:160-244).
 * While a system's positions are those of its last rebin (the rebuild steps of
 * xnb_step, xnb_init_particles, xnb_update_particles_full, and xnb_chunk_neighbors
 * until positions next change), cells with an AMR sub-grid (side 2 or 3) test
 * each sub-cell's particles only against the sub-cells of the 27 neighbour cells
 * whose boxes lie within nbh_dist of it; after positions change, a build without
 * a rebin searches whole cells. The lists are the same either way. */
int xnb_batch_set_subcell_pruning(xnb_batch* b, int32_t on);

/* Changes the launch configuration of a live batch (same limits as at creation). */
int xnb_batch_set_tuning(xnb_batch* b, int32_t stage_cap, int32_t force_block);
/* Online autotuner: coordinate search over the neighbour-build form
 * {ROWS, WARP}, stage_cap {384, 640, 1024}, force_block {64, 128, 256}, force
 * threads per particle {1, 2, 4} and the Newton traversal (the batch's force
 * form is kept), each configuration timed
 * (CUDA events on `stream`) over trial_steps of xnb_step without host sync
 * after one untimed step. The trials are real MD steps: the batch advances
 * (1 + trial_steps) x trials steps. The batch is left on the fastest
 * configuration, which *out describes; precision is the base precision
 * (XNB_PREC_FP64 or XNB_PREC_MIXED) the run will use. Synchronises. */
int xnb_autotune(xnb_batch* b, int32_t trial_steps, int32_t precision, void* stream, xnb_tuning* out);

/* ---- reference-format neighbour streams ---- */

/* chunk_neighbors' own output layout (GridChunkNeighbors::m_cell_stream,
 * chunk_neighbors.h:42-120; encoding of chunk_neighbors_execute.h:249-398 with
 * chunk size 1), so the reference's other pair functors can traverse lists built
 * here. One u16 stream per interior cell of system `sys`, in the grid's linear
 * cell order, concatenated into `stream` (device memory, `cap` u16 entries); cell
 * c's stream is stream[cell_offsets[c] .. cell_offsets[c+1]) (device array of
 * n_cells + 1 u64). offset_tables: 0, 1 (per-particle offsets, the reference's
 * build_particle_offset) or 2 (plus the per-particle count of lower-ordered
 * neighbours, dual_particle_offset). Particle indices in a periodic-image cell
 * number the owner cell's particles that pass the ghost filter, as in the
 * reference's ghost cells. stream == NULL: only the sizes (cell_offsets and
 * *total_out). The lists must describe the current positions (call after
 * xnb_chunk_neighbors / xnb_update_particles_full, before positions change);
 * otherwise XNB_ERR_ARG. XNB_ERR_CAPACITY when *total_out > cap. Synchronises. */
int xnb_chunk_neighbors_stream(xnb_batch* b, int32_t sys, int32_t offset_tables, uint16_t* stream, int64_t cap,
                               uint64_t* cell_offsets, int64_t* total_out, void* cuda_stream);
/* verify_chunk_neighbors (particle_neighbors/verify_chunk_neighbors.cpp:58-168) for
 * streams in the layout above (device pointers; stream_len u16 entries, and a
 * cell whose offsets leave [0, stream_len] counts as a format error), against the
 * current positions:
 * counts_out[6] = format (tables, lengths, reads past a stream), order (cells or
 * indices not increasing, second table wrong), self, range (cell outside the
 * 27-cell block or index past the cell's size), far (listed pair not within
 * 0 < d2 <= nbh_dist^2), missing (per particle, |listed - found| by an exhaustive
 * FP64 search of the 27-cell block with the ghost filter). All zero: the streams
 * hold exactly the reference's neighbour sets. Synchronises. */
int xnb_verify_chunk_neighbors(xnb_batch* b, int32_t sys, int32_t offset_tables, const uint16_t* stream,
                               int64_t stream_len, const uint64_t* cell_offsets, int64_t* counts_out,
                               void* cuda_stream);

/* ---- other pair functors through the same lists ---- */

/* Particle types (the reference's field::type, 0 until set) by id: types[k] for
 * ids[k] (host arrays, n <= 2^24, distinct ids). *matched = particles of the
 * system that were found. Types follow their particles through rebins. */
int xnb_system_set_types(xnb_batch* b, int32_t sys, const uint64_t* ids, const uint8_t* types, int64_t n,
                         int64_t* matched, void* stream);
/* gravitational_force (GravitationalForceFunctor, contribs/pi/gravitational_force.cu:
 * 42-141) over the current neighbour lists: for pairs within rcut (<= the lists'
 * rcut + rcut_inc), f_a += G m_a m_b / r^3 * (r_b - r_a) with masses type_mass[type]
 * (ntypes <= 16). precision XNB_PREC_FP64_EXACT (the functor's own roundings) or
 * XNB_PREC_FP64. flags: XNB_FORCE_ENERGY also writes 0.5 * sum(-G m_a m_b / r) per
 * particle; XNB_FORCE_ACCUMULATE adds onto the current forces (as the reference's
 * buffer-less functors add onto the force field), otherwise forces start at zero
 * (zero_particle_force). A particle type without a mass returns XNB_ERR_ARG. */
#define XNB_FORCE_ENERGY 1
#define XNB_FORCE_ACCUMULATE 2
#define XNB_FORCE_MIXED 4 /* xnb_snap_force: FP32 arithmetic for U, Z, Y and the adjoint */
int xnb_gravitational_force(xnb_batch* b, int32_t sys, double G, const double* type_mass, int32_t ntypes,
                            double rcut, int32_t precision, int32_t flags, void* stream);

/* ---- pair-functor API (include/xnb_pair.cuh) ---- */

/* Device-side view of one resident system for pair functors compiled against
 * include/xnb_pair.cuh: the arrays the traversal of compute_cell_particle_pairs
 * (compute/include/exanb/compute/compute_cell_particle_pairs.h:119-245) reads
 * and writes, over the lists built here. Particles are in storage order
 * (0 .. n_particles-1); a list entry is (particle index << 5) | periodic image
 * code. Pointers are device addresses into the batch's pools: valid until the
 * system is removed or the batch destroyed; positions and lists change with
 * every step and rebuild. */
typedef struct xnb_pair_view {
  int64_t n_particles;
  const double *rx, *ry, *rz;
  double *vx, *vy, *vz;
  double *fx, *fy, *fz;
  double* pe;                /* per-particle energy field */
  const uint64_t* id;
  const uint8_t* type;       /* field::type */
  const void* mirror;        /* float4 per particle: fl32(r - origin) per axis, 0 */
  const void* mirror_lo;     /* float4 per particle: fl32((r - origin) - mirror) per axis, 0 */
  const uint32_t* nbr;       /* the system's list entries */
  const uint32_t* nbr_start; /* per particle: its first entry in nbr */
  const uint32_t* nbr_count; /* per particle: its list length */
  const uint32_t* nbr_half;  /* per particle: entries ahead of the particle itself in the reference's
                                (cell_enc, p_b) order, the lower half of the symmetric split */
  double origin[3];
  double period[3];          /* extent - origin: the periodic image offsets */
  double nbh_dist;           /* rcut + rcut_inc the lists were built with */
  double max_period;         /* largest period (the FP32 prefilter's error bound uses it) */
  double mass;               /* the system's particle mass and its divide_by_mass flag */
  int32_t divide_by_mass;
  int32_t sys;
} xnb_pair_view;
/* Fills *out for system sys (no GPU work). */
int xnb_system_pair_view(xnb_batch* b, int32_t sys, xnb_pair_view* out);

/* ---- on-device observables ---- */

typedef struct xnb_sim_stats {
  int64_t particle_count;
  double kinetic_sum;      /* sum over particles of dot(v, v) * 1.0, as simulation_stats forms it (its mass is 1.0) */
  double potential_energy; /* sum of the per-particle energies of the last force call made with energies */
  double min_vel, max_vel; /* extremes of |v| */
  double min_acc, max_acc; /* extremes of |f| (the force field the reference names ax, ay, az) */
} xnb_sim_stats;

/* simulation_stats (ComputeSimulationStatistics, debug/simulation_stats.cpp:60-124)
 * reduced on the GPU for one system; sums in a fixed order (blocks folded in
 * index order), so repeated calls agree bit for bit. Synchronises. */
int xnb_simulation_stats(xnb_batch* b, int32_t sys, xnb_sim_stats* out, void* stream);
/* Values of chosen particles by id, gathered on the GPU (what check_values,
 * debug/check_values.cpp:230-401, compares): values[k*9 + 0..8] = rx ry rz fx fy fz
 * vx vy vz of ids[k], found[k] = 1 when the id belongs to the system (0 and the
 * values untouched otherwise). Host arrays; n <= 2^24; ids need not be sorted
 * but must be distinct. Synchronises. */
int xnb_sample_particles(xnb_batch* b, int32_t sys, const uint64_t* ids, int64_t n, double* values, int32_t* found,
                         void* stream);

/* ---- allocation-free entry point ---- */

/* No counterpart in the reference. chunk_neighbors for one system, for callers
 * that cannot allocate device memory where they need the lists: a host
 * framework that owns all device memory through its own pools and forbids
 * cudaMalloc inside a step, or a time-stepping loop that must not stall on the
 * device-wide synchronisation cudaFree can impose. It allocates nothing:
 * inputs and outputs are the caller's device buffers, and scratch is one
 * file-scope device array of the library (about 5.3 MB, held by every GPU that
 * loads the library until exit).
 *   rx, ry, rz       n positions in cell order (cells in linear order (k*Dj+j)*Di+i)
 *   cell_start/count per cell: first particle index (0-based) and particle count
 *   nbr              output entries (local index << 5 | periodic image code), in
 *                    the reference's (cell_enc, p_b) order; capacity nbr_capacity
 *   nbr_start/count  output per particle: first entry and number of entries
 *   total_out        entries needed (set also when the capacity is too small)
 * Limits: n <= 1,048,576 particles, <= 131,072 cells (the dims product, checked
 * in 64 bits) and at most 2^32 - 1 entries (a larger nbr_capacity counts as
 * 2^32 - 1); larger inputs return XNB_ERR_ARG with the limit in
 * xnb_last_error_string(). Returns XNB_ERR_CAPACITY when total_out >
 * nbr_capacity (nbr and nbr_start are then left unwritten; nbr_count holds the
 * per-particle counts).
 * The first call on a device looks up the scratch array's address (set-up);
 * make it before any stream capture begins on that device. All calls share the
 * array: calls that overlap on the GPU race and must be serialised by the
 * caller. Each call copies total_out to the host and synchronises `stream`. */
int xnb_chunk_neighbors_noalloc(const xnb_lj_params* p, int64_t n, const double* rx, const double* ry,
                                const double* rz, const uint32_t* cell_start, const uint32_t* cell_count,
                                uint32_t* nbr, int64_t nbr_capacity, uint32_t* nbr_start, uint32_t* nbr_count,
                                int64_t* total_out, void* stream);

/* ---- SNAP (snap_force_generic, contribs/md/snap/include/md/snap/snap_force.h:
 *      134-372) ---- */
/* A linear SNAP potential as the reference reads it from LAMMPS files
 * (lib/snap_read_lammps.cpp:30-132): rcutfac, rfac0, rmin0, twojmax (<= 10),
 * switchflag, bzeroflag; per particle type radelem, the weight wj and
 * ncoeffall coefficients (constant term first, bispectrum order of
 * sna.cpp:236-259). chemflag, bnormflag, quadraticflag, switchinnerflag must be
 * 0 and wselfallflag is irrelevant for one element set. Forces and energies are
 * multiplied by energy_unit (1 eV in the system's units when the coefficients
 * are in eV, as the reference does without conv_coef_units). */
typedef struct xnb_snap_params {
  int32_t twojmax;
  double rcutfac;
  double rfac0;
  double rmin0;
  int32_t switchflag;
  int32_t bzeroflag;
  int32_t chemflag;
  int32_t bnormflag;
  int32_t quadraticflag;
  int32_t switchinnerflag;
  int32_t ntypes; /* <= 16 */
  double radelem[16];
  double wj[16];
  int32_t ncoeffall;
  const double* coeff; /* ntypes x ncoeffall */
  double energy_unit;
} xnb_snap_params;
typedef struct xnb_snap xnb_snap;
/* Builds the potential's tables (Clebsch-Gordan blocks, index lists, the
 * coefficient multipliers of the adjoint) on `device`. */
int xnb_snap_create(const xnb_snap_params* p, int32_t device, xnb_snap** out);
int xnb_snap_destroy(xnb_snap* s);
/* zero_particle_force + snap_force_generic + update_force_from_ghost (+ the
 * division by mass of systems whose force chain ends with it) over the current
 * lists, FP64; with XNB_FORCE_MIXED the U, Z, Y and adjoint arithmetic runs in
 * FP32 while displacements, the Cayley-Klein parameters, the switching
 * function and every force sum stay in FP64 (about 1e-7 relative force error). The SNAP cutoff (rad_a + rad_b) rcutfac must not exceed the
 * lists' rcut + rcut_inc. flags: XNB_FORCE_ENERGY writes the per-particle SNAP
 * energy to pe; XNB_FORCE_ACCUMULATE adds onto the current forces. An
 * environment of more than 128 neighbours or a particle type without
 * coefficients returns XNB_ERR_ARG. Synchronises `stream`. */
int xnb_snap_force(xnb_batch* b, int32_t sys, const xnb_snap* snap, int32_t flags, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* XNB_GPU_H */
