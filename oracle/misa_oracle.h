/*
 * TEST INFRASTRUCTURE - NOT PART OF THE PRODUCT.
 *
 * C API of the CPU oracle: a single-rank restatement of MISA-MD's per-step EAM
 * hot path (src/atom.cpp, src/newton_motion.cpp, src/atom/, src/lattice/,
 * src/pack/, src/system_configuration.cpp, src/simulation.cpp:155-217).
 * Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg may load
 * it, and only as the checker or the timed CPU baseline.
 *
 * The record layout below is the reference's AtomElement
 * (src/atom/atom_element.h:18-41) on an LP64 host: 104 bytes.
 */
#ifndef MISA_ORACLE_H
#define MISA_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct orc_atom {
    uint64_t id;
    int32_t type; /* -1 INVALID (vacancy / moved to the inter-atom list), 0 Fe, 1 Cu, 2 Ni */
    int32_t pad_;
    double x[3];
    double v[3];
    double f[3];
    double rho;
    double df;
} orc_atom;

/* Geometry of one libcomm sub-domain (BccDomain restated). For a simulation the
 * grid is 1x1x1 (one rank, periodic self-exchange). Other grids are only used
 * by the Wigner-Seitz known-answer tests. */
typedef struct orc_domain_desc {
    int64_t phase_space[3];
    double lattice_const;
    double cutoff_radius_factor;
    int32_t grid_size[3];
    int32_t grid_coord[3];
    int32_t ghost_size; /* <= 0: ceil(cutoff_radius_factor) + 1 as src/simulation.cpp:46 */
} orc_domain_desc;

/* ---- Wigner-Seitz helpers on a described domain (src/lattice/ws_utils.cpp) ---- */
void orc_ws_near_lat_sub_box_coord(const orc_domain_desc *d, const double x[3], int64_t out[3]);
void orc_ws_near_lat_coord(const orc_domain_desc *d, const double x[3], int64_t out[3]);
uint32_t orc_ws_is_out_box(const orc_domain_desc *d, const double x[3]);
int64_t orc_ws_find_near_lat_index_in_sub_box(const orc_domain_desc *d, const double x[3]);
/* Batch of n points (xyz interleaved): ghost-extended coords (getNearLatCoord), sub-box coords
 * (getNearLatSubBoxCoord), isOutBox flags and findNearLatIndexInSubBox. Any output may be NULL. */
void orc_ws_batch(const orc_domain_desc *d, const double *xyz, int64_t n, int64_t *ext_coords,
                  int64_t *sub_coords, uint32_t *flags, int64_t *index);

/* ---- neighbour offset tables (src/atom/neighbour_index.inl:13-76) on an explicit slot grid ---- */
/* which: 0 full-even, 1 full-odd, 2 half-even, 3 half-odd. Returns the table length; writes
 * min(len, cap) entries. size_x is doubled. */
int32_t orc_nei_offsets(int64_t size_x, int64_t size_y, int64_t size_z, int32_t cut_lattice,
                        double cutoff_radius_factor, int32_t which, int64_t *out, int32_t cap);
int32_t orc_is_positive_index(double x, double y, double z);

/* ---- simulation state ---- */
typedef struct orc_sim orc_sim;

/* Creates the single-rank simulation on a phase_space box; the potential is read from a setfl file.
 * Returns NULL on error (message via orc_last_error). */
orc_sim *orc_create(const int64_t phase_space[3], double lattice_const, double cutoff_radius_factor,
                    const char *setfl_path, double timestep_ps);
void orc_destroy(orc_sim *s);
const char *orc_last_error(void);

/* Slot grid sizes: size_x (doubled), size_y, size_z, ghost (doubled x), ghost y, ghost z. */
void orc_grid(const orc_sim *s, int64_t out[6]);
int64_t orc_n_slots(const orc_sim *s);

/* Copy the whole lattice slot array (reference linear index order, ghosts included) in/out. */
void orc_set_atoms(orc_sim *s, const orc_atom *atoms, int64_t n);
void orc_get_atoms(const orc_sim *s, orc_atom *atoms, int64_t n);
/* Inter-atom lists (list order). Returns the count; writes min(count, cap). */
int64_t orc_get_inter(const orc_sim *s, orc_atom *out, int64_t cap);
int64_t orc_get_ghost_inter(const orc_sim *s, orc_atom *out, int64_t cap);
void orc_set_inter(orc_sim *s, const orc_atom *in, int64_t n);

void orc_set_timestep(orc_sim *s, double dt_ps);
/* Variable timestep (extension, not in the reference): before each step of orc_simulate,
 * dt = clamp(dx_max / max|v|, dt_min, dt_max) over local lattice and local inter atoms. */
void orc_set_variable_timestep(orc_sim *s, double dx_max, double dt_min_ps, double dt_max_ps);
double orc_max_speed2(orc_sim *s);
/* dt of every step orc_simulate took (returns the count; copies at most cap), and their sum. */
int64_t orc_dt_history(const orc_sim *s, double *out, int64_t cap);
double orc_time(const orc_sim *s);

/* Pieces of one step, in src/simulation.cpp:164-194 order. */
void orc_firststep(orc_sim *s);
int32_t orc_decide(orc_sim *s);
void orc_exchange_inter(orc_sim *s);
void orc_border_inter(orc_sim *s);
void orc_exchange_atom_first(orc_sim *s);
void orc_exchange_atom(orc_sim *s);
void orc_clear_force(orc_sim *s);
void orc_compute_eam(orc_sim *s);
void orc_secondstep(orc_sim *s);

/* prepareForStart body (src/simulation.cpp:137-145): first ghost exchange, clearForce, computeEam. */
void orc_prepare(orc_sim *s);
/* nsteps of the loop body of src/simulation.cpp:164-194 (no stage hooks). */
void orc_simulate(orc_sim *s, int64_t nsteps);
/* collisionStep (src/simulation.cpp:208-217). lat = (cell x, cell y, cell z, basis). */
void orc_collision_step(orc_sim *s, const int32_t lat[4], const double dir[3], double energy_ev);
void orc_setv(orc_sim *s, const int32_t lat[4], const double dir[3], double energy_ev);

/* Thermo (src/system_configuration.cpp). */
/* WorldBuilder::build (src/world_builder.cpp:64-199) into the simulation's slots: rng 0 mt19937,
 * 1 minstd_rand, 2 ranlux24, 3 LegacyRand (the MD_RAND choices); atom types from the C library's
 * rand() in its default state. Returns 0, or 1 for an unknown rng. */
int32_t orc_world_build(orc_sim *s, double t_set, uint32_t seed, const int32_t ratio[3], int32_t rng);
double orc_mvv(const orc_sim *s);
double orc_kinetic_energy(const orc_sim *s);
double orc_temperature(const orc_sim *s, uint64_t n_atoms);
void orc_rescale(orc_sim *s, double t_set, uint64_t n_atoms);
void orc_system_force(const orc_sim *s, double out[3]);
/* Extension (the reference computes no potential energy): per-atom
 * E_i = F(rho_i) + 1/2 sum_j phi_ij, returned summed. Needs a computeEam before. Optionally
 * writes per-slot energies (n_slots doubles; vacancies and ghosts 0) and per-inter energies. */
double orc_potential_energy(orc_sim *s, double *per_slot, double *per_inter, int64_t inter_cap);

/* Potential evaluation (the pot v0.1.0 call sites, restated). key = atomic number. */
double orc_pot_charge_density(const orc_sim *s, int32_t key, double r2);
double orc_pot_d_embed(const orc_sim *s, int32_t key, double rho);
double orc_pot_embed(const orc_sim *s, int32_t key, double rho);
double orc_pot_to_force(const orc_sim *s, int32_t key_i, int32_t key_j, double r2, double df_i, double df_j);
double orc_pot_pair(const orc_sim *s, int32_t key_i, int32_t key_j, double r2);
/* Spline coefficients of one table: kind 0 F(rho), 1 rho(r), 2 r*phi(r); for kind 2 e2 is the
 * second element. Writes 7*n doubles (c0,c1,c2,c3,d0,d1,d2 per knot). Returns n. */
int32_t orc_pot_spline(const orc_sim *s, int32_t kind, int32_t e1, int32_t e2, double *out, int32_t cap);

/* Atom dump records (AtomDump::dump, frontend/io/atom_dump.cpp:59-81; BufferedFileWriter::write,
 * frontend/io/buffered_io.cpp:17-35): the inter atoms in list order, then the sub-box lattice atoms in
 * k, j, i order without INVALID slots; each record {id, step, type, inter_type = 0, x, v}, 72 bytes
 * (the layout tools/dump2text/out_convert.cpp:18-25 reads). Writes min(n, cap); returns n. */
typedef struct orc_dump_record {
    uint64_t id;
    uint64_t step;
    int32_t type;
    int16_t inter_type;
    int16_t pad_;
    double x[3];
    double v[3];
} orc_dump_record;
int64_t orc_dump_records(const orc_sim *s, uint64_t time_step, orc_dump_record *out, int64_t cap);

/* Time nsteps of the loop on this thread; returns wall seconds. */
double orc_time_simulate(orc_sim *s, int64_t nsteps);

#ifdef __cplusplus
}
#endif
#endif
