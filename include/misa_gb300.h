/*
 * misa_gb300: GB300-native (sm_103a) EAM step for MISA-MD's lattice-indexed atom store.
 *
 * C ABI of libmisa_gb300.so. Plain pointers and sizes only; every entry point returns an mg_status
 * (0 = success) and never throws. One context owns one CUDA stream on one GPU; a context is not
 * thread-safe, distinct contexts are independent.
 *
 * The record exchanged with the host is the reference's AtomElement (src/atom/atom_element.h:18-41)
 * on LP64: id u64, type i32 (atom_type: -1 INVALID, 0 Fe, 1 Cu, 2 Ni), 4 bytes padding, then
 * x[3], v[3], f[3], rho, df as doubles: 104 bytes. Slot arrays use the reference's linear index
 * (z * size_y + y) * size_x + x over the ghost-extended grid with doubled x
 * (src/lattice/lattice.h:63-66, src/atom/atom_set.cpp:18-26).
 */
#ifndef MISA_GB300_H
#define MISA_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct mg_atom_element {
    uint64_t id;
    int32_t type;
    int32_t pad_;
    double x[3];
    double v[3];
    double f[3];
    double rho;
    double df;
} mg_atom_element;

typedef int32_t mg_status;
enum {
    MG_OK = 0,
    MG_ERR_ARG = 1,          /* bad argument (null pointer, size mismatch, unsupported box) */
    MG_ERR_CUDA = 2,         /* a CUDA runtime call failed; see mg_last_error */
    MG_ERR_POTENTIAL = 3,    /* setfl file missing or malformed, or potential not initialised */
    MG_ERR_CAPACITY = 4,     /* inter-atom or ghost inter-atom list overflowed its capacity */
    MG_ERR_OUT_OF_GRID = 5,  /* an index left the ghost-extended slot grid (atom too far out of the box) */
    MG_ERR_STATE = 6         /* call out of order (e.g. simulate before prepare) */
};

enum { MG_PREC_FP64 = 0, MG_PREC_MIXED = 1 };

/* Device-side error bits reported by mg_thermo / mg_last_device_error. */
enum {
    MG_DEVERR_INTER_OVERFLOW = 1,
    MG_DEVERR_GHOST_OVERFLOW = 2,
    MG_DEVERR_OUT_OF_GRID = 4,
    MG_DEVERR_DISPLACED_OVERFLOW = 8,
    MG_DEVERR_BAD_TYPE = 16
};

typedef struct mg_context mg_context;

/* ---------------------------------------------------------------------------------------------
 * Environment: replaces cuda_env_init / cuda_env_clean (src/arch/arch_imp.h:17-19, called from
 * src/arch/arch_env.hpp:15-25). Selects the device for contexts created afterwards.
 * ------------------------------------------------------------------------------------------- */
mg_status mg_env_init(int32_t device);
mg_status mg_env_clean(void);

/* ---------------------------------------------------------------------------------------------
 * Context: replaces cuda_domain_init(const comm::BccDomain*) (src/arch/arch_imp.h:21, called at
 * src/simulation.cpp:52-54). One rank owning the whole periodic box: phase_space unit cells per
 * dimension, ghost width ceil(cutoff_radius_factor)+1 (src/simulation.cpp:46), cutoff radius
 * lattice_const * cutoff_radius_factor (src/atom.cpp:14-19). Every dimension must be at least
 * 2 * ghost cells. precision: MG_PREC_FP64 or MG_PREC_MIXED. inter_capacity: maximum local
 * inter-atom count (0 picks a default).
 * ------------------------------------------------------------------------------------------- */
mg_status mg_create(const int64_t phase_space[3], double lattice_const, double cutoff_radius_factor,
                    int32_t precision, int64_t inter_capacity, mg_context **out);
mg_status mg_destroy(mg_context *ctx);
/* Last error message of the context (or of the last failed mg_create when ctx is NULL). */
const char *mg_last_error(const mg_context *ctx);
/* Slot grid: size_x (doubled), size_y, size_z, ghost_x (doubled), ghost_y, ghost_z. */
mg_status mg_grid(const mg_context *ctx, int64_t out[6]);
mg_status mg_set_precision(mg_context *ctx, int32_t precision);

/* ---------------------------------------------------------------------------------------------
 * Neighbour offsets: replaces cuda_nei_offset_init(const NeighbourIndex<AtomElement>*)
 * (src/arch/arch_imp.h:23, called at src/simulation.cpp:67-69). The context builds its own
 * tables at mg_create; this entry point checks the host's four tables against them (same entries,
 * same order) and returns MG_ERR_ARG on any difference.
 * ------------------------------------------------------------------------------------------- */
mg_status mg_nei_offset_init(mg_context *ctx, const int64_t *full_even, const int64_t *full_odd, int32_t n_full,
                             const int64_t *half_even, const int64_t *half_odd, int32_t n_half);
/* Copies one of the context's tables out (which: 0 full-even, 1 full-odd, 2 half-even, 3 half-odd,
 * 4 pruned-full-even, 5 pruned-full-odd). Returns the table length in *n. */
mg_status mg_nei_offsets(const mg_context *ctx, int32_t which, int64_t *out, int32_t cap, int32_t *n);

/* ---------------------------------------------------------------------------------------------
 * Potential: replaces cuda_pot_init(eam*) (src/arch/arch_imp.h:25, called at src/simulation.cpp:133
 * after interpolateFile). Either a setfl file, or the parsed tables (F[e][nrho], rho[e][nr],
 * r*phi[pair][nr] for pairs i>=j in lower-triangle order). atomic_numbers map atom types
 * Fe/Cu/Ni (keys 26/29/28, src/types/atom_types.h:61-73) to table elements.
 * ------------------------------------------------------------------------------------------- */
mg_status mg_pot_init_setfl(mg_context *ctx, const char *path);
mg_status mg_pot_init_tables(mg_context *ctx, int32_t n_ele, const int32_t *atomic_numbers, int32_t nrho,
                             double drho, int32_t nr, double dr, double cutoff, const double *F_tables,
                             const double *rho_tables, const double *rphi_tables);
/* Spline coefficients the context uses for one table (kind 0 F, 1 rho, 2 r*phi of pair (e1,e2)):
 * 7 doubles per knot (c0, c1, c2, c3, d0, d1, d2). Returns the knot count in *n. */
mg_status mg_pot_spline(const mg_context *ctx, int32_t kind, int32_t e1, int32_t e2, double *out, int32_t cap,
                        int32_t *n);

/* ---------------------------------------------------------------------------------------------
 * The reference's per-phase accelerator hooks (src/arch/arch_imp.h:27-31), called from
 * atom::latRho / latDf / latForce (src/atom.cpp:159-160, 293-294, 320-321) with the host AoS slot
 * array of the whole ghost-extended grid. On return the host array holds:
 *   rho_calc:   rho of every local slot = the full lattice-lattice density (periodic images
 *               included); ghost-slot rho is left 0, so the reverse rho fold that follows adds 0.
 *   df_calc:    df = F'(rho) of every local non-vacancy slot.
 *   force_calc: f of every local slot = the full lattice-lattice force (ghost-slot f left 0).
 * Ghost df must already hold the owners' df (the host's forward df exchange runs before
 * force_calc, src/atom.cpp:123-137). cutoff_radius must equal the context's cutoff.
 * ------------------------------------------------------------------------------------------- */
mg_status mg_eam_rho_calc(mg_context *ctx, mg_atom_element *atoms, double cutoff_radius);
mg_status mg_eam_df_calc(mg_context *ctx, mg_atom_element *atoms, double cutoff_radius);
mg_status mg_eam_force_calc(mg_context *ctx, mg_atom_element *atoms, double cutoff_radius);

/* ---------------------------------------------------------------------------------------------
 * Resident state: the whole step of simulation::simulate (src/simulation.cpp:164-194) on the GPU,
 * state kept in HBM between calls.
 * ------------------------------------------------------------------------------------------- */
/* Upload the slot array (n_slots records, reference index order) and the inter-atom list. */
mg_status mg_upload(mg_context *ctx, const mg_atom_element *atoms, int64_t n_slots, const mg_atom_element *inter,
                    int64_t n_inter);
/* Download the slot array and the inter-atom list (list order); *n_inter receives the count. */
mg_status mg_download(mg_context *ctx, mg_atom_element *atoms, int64_t n_slots, mg_atom_element *inter,
                      int64_t inter_cap, int64_t *n_inter);
/* Ghost inter atoms (type, x, df; other fields 0), list order. */
mg_status mg_download_ghost_inter(mg_context *ctx, mg_atom_element *ghost, int64_t cap, int64_t *n_ghost);
/* NewtonMotion::setTimestepLength (src/newton_motion.cpp:13-17), dt in ps. Fixed dt from the next step. */
mg_status mg_set_timestep(mg_context *ctx, double dt_ps);
/* Variable timestep (extension; the reference changes dt only per stage, frontend/md_simulation.cpp:42-58).
 * Before each step, dt = clamp(dx_max / max|v|, dt_min, dt_max), max over local lattice and inter atoms,
 * computed on the device as (vx^2 + vy^2) + vz^2, sqrt, divide, each correctly rounded. Units: Angstrom,
 * ps. mg_set_timestep returns to a fixed dt. */
mg_status mg_set_variable_timestep(mg_context *ctx, double dx_max, double dt_min_ps, double dt_max_ps);
/* Steps taken since creation, simulated time (sum of the dt used) and the dt of the last step. Syncs. */
mg_status mg_clock(mg_context *ctx, int64_t *steps, double *time_ps, double *dt_ps);
/* The dt of the most recent min(steps, cap, 65536) steps, oldest first; *n_out = how many. Syncs. */
mg_status mg_dt_history(mg_context *ctx, double *out, int64_t cap, int64_t *n_out);
/* simulation::prepareForStart body (src/simulation.cpp:137-145): first ghost exchange, computeEam. */
mg_status mg_prepare(mg_context *ctx);
/* nsteps iterations of the loop body (src/simulation.cpp:165-193): firststep, decide, exchangeInter,
 * borderInter, exchangeAtom, computeEam, secondstep. Asynchronous on the context stream unless
 * sync != 0. The step sequence is captured once as a CUDA graph and replayed; in the mixed form with
 * a fixed dt, runs of 16 bodies replay one fused graph (mg_set_step_fusion). */
mg_status mg_simulate(mg_context *ctx, int64_t nsteps, int32_t sync);
/* One phase of the loop body, for parity checks: 0 firststep, 1 decide, 2 exchangeInter,
 * 3 borderInter, 4 exchangeAtom, 5 computeEam, 6 secondstep. */
mg_status mg_phase(mg_context *ctx, int32_t phase);
/* simulation::collisionStep (src/simulation.cpp:208-217): atom::setv on the slot at
 * lat = (cell x, cell y, cell z, basis) (src/atom.cpp:475-494), exchanges, computeEam. */
mg_status mg_collision_step(mg_context *ctx, const int32_t lat[4], const double dir[3], double energy_ev);
/* configuration::rescale (src/system_configuration.cpp:86-111) with n_atoms for the degrees of freedom. */
mg_status mg_rescale(mg_context *ctx, double t_set, uint64_t n_atoms);

typedef struct mg_thermo_out {
    double mvv;               /* sum m v^2 (src/system_configuration.cpp:61-84) */
    double kinetic_energy;    /* mvv / 2 */
    double potential_energy;  /* sum F(rho_i) + 1/2 sum phi_ij (extension; only when requested) */
    double force_sum[3];      /* configuration::systemForce (src/system_configuration.cpp:8-24) */
    int64_t n_inter;          /* local inter atoms */
    int64_t n_ghost_inter;
    int64_t n_vacancy;        /* INVALID local slots */
    uint32_t device_errors;   /* MG_DEVERR_* bits accumulated since the last mg_clear_errors */
    uint32_t pad_;
} mg_thermo_out;
/* Synchronises the stream. with_energy != 0 runs the per-atom energy pass (needs a preceding
 * computeEam on the current positions, which mg_prepare / mg_simulate / mg_collision_step give). */
mg_status mg_thermo(mg_context *ctx, int32_t with_energy, mg_thermo_out *out);
/* Per-slot energies (n_slots doubles, 0 for vacancies and ghosts) and per-inter energies, from the
 * last energy pass. */
mg_status mg_download_energies(mg_context *ctx, double *per_slot, int64_t n_slots, double *per_inter,
                               int64_t inter_cap);
mg_status mg_clear_errors(mg_context *ctx);

/* ---------------------------------------------------------------------------------------------
 * Drop-in full step with host state (the end-to-end path): uploads the host slot array and
 * inter-atom list, runs nsteps loop bodies on the GPU, downloads both back. The host arrays keep
 * being the state of record, as in the reference's host loop. Device errors of the step are
 * returned (MG_ERR_CAPACITY, ...).
 * One loop body with a fixed dt and no inter atoms in (*n_inter == 0) is pipelined: the slot array
 * moves in z-chunks of whole planes. In boxes of at least 24 planes the density and force slabs run
 * as their planes arrive and go back out while later chunks still come in. Decide is taken per chunk
 * for displaced atoms that return to their own site; any other displaced atom makes the call run the
 * loop body again in full from its kept input (an extra device copy of the slot array). Thinner boxes
 * overlap the copies in with firststep and the copies out with the force slabs. The result is
 * bit-identical to the unpipelined path. With a pinned slot array (mg_host_register) the copies run
 * asynchronously.
 * ------------------------------------------------------------------------------------------- */
mg_status mg_step_host(mg_context *ctx, mg_atom_element *atoms, int64_t n_slots, mg_atom_element *inter,
                       int64_t inter_cap, int64_t *n_inter, int64_t nsteps);
/* Loop bodies per CUDA graph launch of mg_simulate in the mixed form with a fixed dt (default 16; 0 or
 * 1: one body per launch). Inside a launch, each force pass but the last also takes the next body's
 * firststep for its atoms (when no inter atoms exist; the kernels check on the device), which saves
 * the separate firststep pass. The state between launches is the end of a loop body as always, and
 * results are bit-identical either way. mg_run_stages uses the same graph for runs of bodies with
 * no stage event between them. */
mg_status mg_set_step_fusion(mg_context *ctx, int32_t steps_per_graph);
/* Number of z-chunks of mg_step_host's pipeline (default 16; 0 or 1: no pipelining). */
mg_status mg_set_host_pipeline(mg_context *ctx, int32_t chunks);
/* Verlet skin of the mixed form's candidate lists, in Angstrom (default 0.2; 0: off; at most a0).
 * Each group of 32 sites keeps the pruned candidates that some site of the group had within
 * rc + skin when the list was built. The density pass then visits only those, until the sum of the
 * per-step maximum displacements, doubled, reaches the skin; a record written by an upload or by
 * recombination also forces a rebuild. Every pair inside the cutoff is visited either way, in the
 * same order, so results are bit-identical for every skin. Captured graphs are rebuilt. */
mg_status mg_set_neighbour_skin(mg_context *ctx, double skin);
/* Density passes that used the mixed form's candidate lists, and how many of them rebuilt the lists
 * (diagnostics). Syncs. */
mg_status mg_skin_stats(mg_context *ctx, int64_t *passes, int64_t *rebuilds);

/* ---------------------------------------------------------------------------------------------
 * Wigner-Seitz mapping on the GPU (src/lattice/ws_utils.cpp:91-189), for indexing parity checks:
 * for n positions (xyz interleaved) writes the ghost-extended nearest-site coordinates
 * (3 int64 per point, doubled x), the box flags of ws::isOutBox and the sub-box linear index of
 * ws::findNearLatIndexInSubBox (-1 when outside).
 * ------------------------------------------------------------------------------------------- */
mg_status mg_ws_map(mg_context *ctx, const double *xyz, int64_t n, int64_t *coords, uint32_t *flags,
                    int64_t *index);

/* Autotuner: times the density and force passes of the current precision on the resident state for
 * every gather thread order (0: all even sites then all odd; 1: even/odd warps interleaved per 32
 * sites), block size (128, 256, 512) and number of sites per thread (1, 2, 4; a thread's sites are
 * one grid stride apart), reps launches each, and keeps the fastest. Results are cached per
 * (box, precision) for the life of the process. out (may be NULL) receives {rho order, rho block,
 * rho sites per thread, force order, force block, force sites per thread}. Needs mg_prepare first. */
mg_status mg_autotune(mg_context *ctx, int32_t reps, int32_t out[6]);
/* Sets the six tuning values directly (same layout as mg_autotune's out). */
mg_status mg_set_tuning(mg_context *ctx, const int32_t tune[6]);

/* Measured kernel times of the last mg_simulate call with timing enabled (ms per step per kernel). */
mg_status mg_enable_timing(mg_context *ctx, int32_t on);
mg_status mg_kernel_times(const mg_context *ctx, double *ms, int32_t cap, int32_t *n, const char **names);
/* Number of kernel launches per loop-body step in the captured graph. */
mg_status mg_launches_per_step(const mg_context *ctx, int32_t *n);
/* CUDA stream of the context (a cudaStream_t), for callers timing on it. */
void *mg_stream(const mg_context *ctx);

/* ---- Stage machine (MDSimulation::beforeStep / postStep, frontend/md_simulation.cpp:40-111) ----
 * Runs `steps` loop bodies through a list of stages as the reference's driver does: when the current
 * stage's steps are used up (checked once per step), the next stage starts and sets its dt
 * (step_length 0: default_dt); a stage with collision_set applies its PKA (simulation::collisionStep)
 * before stage step collision_step - 1 (the reference does so only when an origin dump path is
 * configured); a stage with rescales_set rescales to rescale_t every rescale_every stage steps
 * (configuration::rescale, n_atoms global atoms). Everything is enqueued on the context's stream;
 * the host waits once, at the end. Every thermo_interval steps (0: none) one sample is recorded:
 * steps taken since creation, simulated time, sum m v^2 and temperature (configuration::temperature).
 * Running out of stages returns MG_ERR_STATE (the reference aborts). */
typedef struct mg_stage {
    int64_t steps;
    double step_length;       /* ps; 0 = default_dt */
    int32_t collision_set;
    int32_t rescales_set;
    int64_t collision_step;   /* 1-based stage step of the collision */
    int32_t collision_lat[4]; /* unit cell x, y, z and basis (0 corner, 1 centre) */
    double direction[3];
    double pka_energy;        /* eV */
    double rescale_t;         /* K */
    int64_t rescale_every;
} mg_stage;
typedef struct mg_thermo_sample {
    int64_t step;
    double time_ps;
    double mvv;
    double temperature;
} mg_thermo_sample;
mg_status mg_run_stages(mg_context *ctx, const mg_stage *stages, int32_t n_stages, int64_t steps, double default_dt,
                        int64_t n_atoms, int32_t thermo_interval, mg_thermo_sample *samples, int64_t cap,
                        int64_t *n_samples);

/* ---- Batched independent replicas (extension, no reference counterpart: the reference runs one
 * simulation per MPI job). One CUDA graph holds the loop body (mg_simulate's step) of every context
 * as its own branch, steps_per_launch bodies deep, so one graph launch advances all replicas; their
 * small kernels (inter-atom list, PKA region) overlap instead of running back to back. Boxes,
 * precisions and timestep rules may differ per replica; every context must be prepared, and must
 * outlive the batch. Work a caller issues on a member context is ordered before or after
 * mg_batch_run as the calls are made. A member whose precision, tuning or potential changed is
 * recaptured at the next run. ---- */
typedef struct mg_batch mg_batch;
mg_status mg_batch_create(mg_context *const *ctxs, int32_t n, int32_t steps_per_launch, mg_batch **out);
/* nsteps loop bodies of every replica; sync != 0 waits and reports the first replica whose device
 * error word is set (message via mg_batch_last_error). */
mg_status mg_batch_run(mg_batch *b, int64_t nsteps, int32_t sync);
/* graph nodes per step of all replicas together */
mg_status mg_batch_launches_per_step(const mg_batch *b, int32_t *n);
void *mg_batch_stream(const mg_batch *b);
const char *mg_batch_last_error(const mg_batch *b);
mg_status mg_batch_destroy(mg_batch *b);

/* ---- Creation mode (simulation::createAtoms with create_mode, src/simulation.cpp:58-85 ->
 * WorldBuilder::build, src/world_builder.cpp:64-199), host only ----
 * Fills a host slot array (n_slots = the grid of mg_grid for this box) with the reference's
 * created crystal: ids 1..N in k, j, i order, types drawn with the C library's rand() in its
 * default state against alloy_ratio (Fe, Cu, Ni), positions on the BCC sites, velocities
 * (u - 0.5) / m from md_rand's engine seeded with seed, zero total momentum, then rescaled to t_set
 * (t_set == 0: no rescale). rng selects the engine the reference build chose with MD_RAND. */
enum { MG_RNG_MT = 0, MG_RNG_LCG = 1, MG_RNG_STC = 2, MG_RNG_LEGACY = 3 };
mg_status mg_world_build(const int64_t phase_space[3], double lattice_const, double cutoff_radius_factor,
                         double t_set, uint32_t seed, const int32_t alloy_ratio[3], int32_t rng,
                         mg_atom_element *atoms, int64_t n_slots);

/* ---- Atom dump (AtomDump::dump / writeDumpHeader, frontend/io/atom_dump.cpp:38-82; OutputCopy,
 * frontend/io/output_copy.cpp:19-59; records as BufferedFileWriter::write,
 * frontend/io/buffered_io.cpp:17-35) ----
 * Binary frames in the copy-mode file layout that tools/dump2text/out_convert.cpp:66-98 reads for
 * one rank: a 128-byte file header (kiwi::LocalStorage's own; no reader uses it, written as zeros),
 * a 128-byte rank header whose first 8 bytes hold the number of records in the file, then the
 * 72-byte records. A frame holds the context's inter atoms in list order, then the lattice atoms of
 * the box in k, j, i order without vacant slots, each with the time step given; inter_type is 0 for
 * every record, as the reference writes it.
 *   by_frame == 0: one file at path; frames are appended and mg_dump_close writes the header
 *                  (OutputCopy without by_frame).
 *   by_frame != 0: path holds "{}", replaced by the time step of each frame; one file per frame,
 *                  each with its header (output_copy.cpp:28-33).
 * A frame is packed on the device (ordered compaction) into one of two staging buffers; a writer
 * thread copies it through two pinned chunks of chunk_bytes (0: 64 MiB) and writes chunk k while
 * chunk k + 1 is in flight. mg_dump_frame returns once the frame is enqueued on the context's stream;
 * it waits only while both staging buffers still hold unwritten frames. A dump belongs to one
 * context: close it (or detach it from the stage machine) before destroying the context. ---- */
typedef struct mg_dump_record {
    uint64_t id;
    uint64_t step;
    int32_t type;
    int16_t inter_type;
    int16_t pad_;
    double x[3];
    double v[3];
} mg_dump_record;
typedef struct mg_dump mg_dump;
mg_status mg_dump_open(mg_context *ctx, const char *path, int32_t by_frame, int64_t chunk_bytes, mg_dump **out);
mg_status mg_dump_frame(mg_dump *d, uint64_t time_step);
/* Waits for every frame, writes the header, closes the file and frees d (also after an error).
 * *records (may be NULL): records written (single file: the header's count; by_frame: all frames).
 * An I/O or CUDA failure of any frame is returned here and by the next mg_dump_frame. */
mg_status mg_dump_close(mg_dump *d, uint64_t *records);
const char *mg_dump_last_error(const mg_dump *d);
/* Dumps of the stage machine (MDSimulation::beforeStep / postStep, frontend/md_simulation.cpp:64-70,
 * 86-90): mg_run_stages appends a frame to `frames` (NULL: none) after every step whose 1-based
 * number is a multiple of interval, with that number as its time step, and before each collision
 * writes the state to origin_path (NULL or "": none) as a one-frame file whose time step is the
 * 0-based number of the step about to run (OutputCopy::beforeCollision). */
mg_status mg_set_stage_output(mg_context *ctx, mg_dump *frames, uint64_t interval, const char *origin_path);

/* Page-lock a host range (the caller's slot array) so mg_step_host / mg_upload / mg_download copy it
 * by DMA; undo with mg_host_unregister before freeing it. */
mg_status mg_host_register(void *ptr, uint64_t bytes);
mg_status mg_host_unregister(void *ptr);

/* Arithmetic-pipe probe (measurement; no reference counterpart): FMA throughput of the current device
 * in FLOP/s (2 per FMA) for kind 0 FP64, 1 FP32, 2 packed FP32x2 (fma.rn.f32x2). Every SM runs
 * independent FMA chains; one warm-up launch, then one launch timed with CUDA events. */
mg_status mg_probe_fma(int32_t kind, double *flops_per_s);

/* ---------------------------------------------------------------------------------------------
 * Sum of m v^2 over n atoms without allocating device memory. No counterpart in the reference:
 * it exists for callers that cannot call cudaMalloc (a host loop running under CUDA-graph capture,
 * a plugin whose host process owns all device memory, a real-time loop that must not block in the
 * allocator); mg_thermo computes the same sum but needs a context, which allocates.
 *   vx, vy, vz: device arrays of n velocities (A/ps); type: device array of n atom types
 *   (-1 vacancy, skipped; 0 Fe, 1 Cu, 2 Ni; the array is not validated, and any other value counts
 *   as mass 0); out_mvv: device pointer to one double receiving sum m v^2 (amu A^2/ps^2); stream:
 *   a cudaStream_t (NULL for the default stream). Asynchronous.
 * At most 33,554,432 atoms (MG_ERR_ARG beyond, message via mg_last_error(NULL)). The partial sums
 * live in a fixed 64 KiB __device__ array that every GPU loading the library keeps until exit and
 * that all calls on a GPU share: calls that overlap on the GPU (two streams at once) race on it.
 * A call on a stream that is not being captured looks up the array's address on the current device
 * (again after a device reset); a call on a capturing stream reuses that address, so make one call
 * on each device before any stream capture begins (MG_ERR_STATE otherwise).
 * ------------------------------------------------------------------------------------------- */
mg_status mg_mvv_noalloc(const double *vx, const double *vy, const double *vz, const int8_t *type, int64_t n,
                         double *out_mvv, void *stream);

#ifdef __cplusplus
}
#endif
#endif
