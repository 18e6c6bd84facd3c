// Internal declarations shared by the misa_gb300 translation units (host + device).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "../../include/misa_gb300.h"

namespace mg {

constexpr int kInvalid = -1;                 // atom_type::INVALID (src/types/atom_types.h:27)
constexpr double kBoltz = 8.617343e-5;       // src/types/pre_define.h:11
constexpr double kMvv2e = 1.0364269e-4;      // src/types/pre_define.h:18
constexpr double kFtm2v = (1.0 / kMvv2e);    // src/types/pre_define.h:19
constexpr double kNeiLatCutoff = 0.5;        // src/md_building_config.h.in:24
constexpr int kMaxFull = 232;                // capacity of a full offset table per parity
constexpr int kFirstThreads = 256;           // firststep block = one group of displaced flags (8 per lane)
constexpr int kSortSmemKeys = 16384;         // bucket keys the list manager sorts in shared memory
constexpr int kListWords = 4;                // list bits per 32-site group: pruned candidates up to 128
constexpr int kSkinSlots = 64;               // words the per-step maximum displacement is spread over

// box flags (src/lattice/box.h:12-20)
constexpr uint32_t kInBox = 0, kXLow = 1u, kXHigh = 2u, kYLow = 4u, kYHigh = 8u, kZLow = 16u, kZHigh = 32u;

// device counters / flags word indices
// CNT_DISP_RAW: displaced slots counted by firststep this step (0 lets the collection kernels skip)
// CNT_TOUCHED: lattice owners listed by an inter-atom pass for the ordered owner gather that follows;
// CNT_TOUCH_DONE: blocks of that gather finished (the last one resets both words)
// CNT_SPEC_VOID: the overlapped host step met a displaced atom whose decide it cannot take per chunk
enum {
    CNT_INTER = 0, CNT_GHOST = 1, CNT_DISPLACED = 2, CNT_ERRORS = 3, CNT_FAR = 4, CNT_DISP_RAW = 5, CNT_TOUCHED = 6,
    CNT_TOUCH_DONE = 7, CNT_SPEC_VOID = 8, CNT_WORDS = 9
};

inline double atom_mass(int type) {  // src/types/atom_types.h:42-53
    switch (type) {
        case 0: return 55.845;
        case 1: return 63.546;
        case 2: return 58.6934;
        default: return 0;
    }
}
inline int type_key(int type) {  // src/types/atom_types.h:61-73
    switch (type) {
        case 0: return 26;
        case 1: return 29;
        case 2: return 28;
        default: return 0;
    }
}

// Slot grid of one rank owning the whole periodic box. x is doubled (even = cube corner,
// odd = body centre); linear index (z * Sy + y) * Sx + x.
struct Geom {
    int Sx, Sy, Sz;          // ghost-extended slot grid
    int gx, gy, gz;          // ghost widths (gx doubled)
    int bx, by, bz;          // box sizes (bx doubled)
    int n_slots, n_local, n_ghost_slots;
    int half;                // n_slots / 2: start of the odd half of the parity-split layout
    int nxh;                 // bx / 2: sites of one parity per row
    int n_local_half;        // n_local / 2
    int cells[3];            // phase space in unit cells
    double a0;               // lattice constant (Angstrom)
    double rc, rc2;          // cutoff radius and its square
    double thr;              // pow(0.2 a0, 2): displacement threshold of atom::decide
    double L[3];             // periodic lengths
    double inv_h;            // 2 / a0: inverse of the half lattice constant
    double inv_a0;           // RN(1 / a0): the Voronoi search's estimate of the quotient x / a0
    float inv_h_f;           // 2 / a0 (float)
    float thr_lo_f;          // thr * (1 - 1e-4) in float: FP32 distances below it skip the exact test
    float h_f;               // a0 / 2 (float)
    float rc2_h;             // (rc / h)^2 in half-lattice units
    float rc2_pre;           // rc2_h * (1 + 1e-4): FP32 candidate test of the FP64 gathers
    float skin_h;            // Verlet skin of the group candidate lists, half-lattice units (0: off)
    float rcs2_h;            // ((rc + skin) / h)^2 (rc2_h when the skin is off)
    // site_half[m] = RN((m / 2) a0), m in [0, n_site_half): the coordinate of half-lattice index m,
    // rounded as the site formula of decide rounds it (x: m = i; y, z: m = 2j + parity)
    const double *site_half;
    int n_site_half;
};

// Verlet skin on the group candidate lists (mixed form). The density pass of some step built the
// lists from the displacement records of that step. Until `dirty` is set, no record has changed since
// then except through firststep (or through recombination, whose neighbourhood marks make the groups
// that can see the atom rebuild their own lists), and every change of a record is at most the
// maximum change of its step (the step_max2 words); acc sums those maxima since the build. A pair
// inside rc now was therefore inside rc + 2 acc when the lists were built, and while 2 acc stays
// below the skin the lists hold every pair inside the cutoff.
struct SkinState {
    unsigned step_max2[kSkinSlots];  // this step's max |du|^2 (float bits, half-lattice units)
    float acc;                       // the sum of the per-step maxima of |du| since the build
    int dirty;                       // a record changed outside firststep: the next pass rebuilds
    int rebuilt;                     // the last density pass rebuilt every group's list
    int pad;
    unsigned long long rebuilds;     // density passes that rebuilt every group's list
    unsigned long long passes;       // density passes with the group lists
};

// Lattice slot arrays (structure of arrays over every slot, ghosts included).
struct Slots {
    double *x, *y, *z;
    double *vx, *vy, *vz;
    double *fx, *fy, *fz;
    double *rho, *df;
    double *e;               // per-atom energy (energy pass only)
    int8_t *type;
    uint64_t *id;
    // mixed form, parity-split layout (slot s at (s & 1) * half + (s >> 1)):
    float4 *u4;              // displacement from the site in half-lattice units, w = type bits
    float4 *u4n;             // the next loop body's u4 buffer when the force pass takes the next firststep
    unsigned *near;          // per 32-site group and parity: kListWords words, the pruned candidates some
                             // site of the group had inside rc + skin when the list was last built
    SkinState *skin;
    float *df32;             // F'(rho) in float
};

// Inter-atom lists (local list in list order; ghost list in receive order).
struct Inter {
    int cap, gcap;
    int *cnt;                // CNT_* words
    uint64_t *id;
    int *type;
    double *x, *y, *z, *vx, *vy, *vz, *fx, *fy, *fz, *rho, *df, *e;
    // ghost inter atoms
    int *gtype, *groot;      // groot: index of the local inter atom this ghost is an image of
    double *gx, *gy, *gz, *gdf;
    // scratch for compaction / sorting (size cap + gcap)
    int *scratch_i;          // 3 * cap
    double *scratch_d;       // 13 * cap
    uint64_t *scratch_u;     // cap
    // displaced lattice slots found by the decide scan, in scan order
    int *displaced;
    int dcap;
    int8_t *dflag;           // per local slot (k, j, i order, padded to whole firststep blocks): 1 = displaced
    int *dblock;             // per firststep block: displaced count, then its exclusive offset
    // per-slot claim word for recombination (INT_MAX when free)
    int *claim;
    // lattice atoms farther than 0.2 a0 from their site (only recombined atoms after decide): they
    // and every atom within their full neighbourhood gather over the whole offset table
    int *far_list;
    int8_t *far_flag;        // per slot: 1 for far atoms and their neighbourhoods
    int fcap;
    // buckets: sorted (key, ref) pairs; ref < cap: local index, else cap + ghost index
    long long *bucket;       // (key << 32) | ref packed, sorted ascending
    int *n_bucket;
    // lattice owners with an inter atom inside the cutoff: one bit per slot (all clear between
    // passes) and the list of owners whose bit an inter-atom pass set, in any order; the owner
    // gather that follows sums each owner's inter-atom terms in a fixed order and clears the bits
    unsigned *touch_bits;
    int *touched;
    int tcap;
};

// One FP64 spline knot record (32 bytes, read as two 16-byte loads).
struct alignas(32) Knot64 {
    double a, b, c, d;
};

// Spline tables on the device. Value records {c0,c1,c2,c3}; derivative records {d0,d1,d2,0}.
// Laid out by atom type (3 tables of nr or nrho knots) and by type pair (9 tables, ti * 3 + tj),
// so a lookup is pointer arithmetic on the type, with no per-lane indexed parameter load.
struct PotTables {
    int nr, nrho;
    double inv_dr, inv_drho;
    float inv_dr_f, inv_drho_f, h_inv_dr_f;   // h_inv_dr_f = (a0/2) / dr
    const Knot64 *rho_v, *rho_d, *F_v, *F_d, *z_v, *z_d;
    const float4 *rho_vf, *rho_dff, *F_vf, *F_dff, *z_vf, *z_dff;
    // force pass, mixed form: per type pair (ti * 3 + tj) and knot one 32-byte record
    // {r*phi c0, rho_tj' d0, c1, d1, c2, d2, c3, 0}; r*phi' comes from the value coefficients
    const float *zr8;
};

// Per-step parameters, resident in device memory (one record per context). Kernels read dt and the
// half-kick factors dt/(2m) from here, so a new timestep needs no new graph. In variable-timestep
// mode the step-head kernel rewrites them every step from the largest speed the previous kick left.
constexpr int kVmaxSlots = 1024;    // spread max-words: one per (warp index mod kVmaxSlots)
constexpr int kDtHistory = 65536;   // ring of the most recent timesteps
struct StepParams {
    double dt;
    double dt_inv_m[3];
    double dx_max, dt_min, dt_max;  // variable timestep: dt = clamp(dx_max / max|v|, dt_min, dt_max); dx_max <= 0: fixed
    double time;                    // simulated time (ps) summed over the steps taken
    long long steps;                // steps taken since the context was created
    long long pad_;
    unsigned long long vmax2[kVmaxSlots];  // max |v|^2 of the last kick, bit patterns of non-negative doubles
    double hist[kDtHistory];               // dt of step k (0-based) at hist[k % kDtHistory]
};

// Host-side spline (FP64 coefficients), built identically to the setfl interpolation scheme.
struct HostSpline {
    int n = 0;
    double delta = 0, inv_delta = 0;
    std::vector<double> c0, c1, c2, c3, d0, d1, d2;
    void build(const std::vector<double> &f, double dlt);
};

struct HostPotential {
    int n_ele = 0;
    std::vector<int> z;
    int nrho = 0, nr = 0;
    double drho = 0, dr = 0, cutoff = 0;
    std::vector<HostSpline> F, rho, z2;   // z2 lower-triangle pair order
    static int pair_index(int a, int b) {
        if (a < b) { int t = a; a = b; b = t; }
        return a * (a + 1) / 2 + b;
    }
    int ele(int key) const {
        for (int i = 0; i < n_ele; i++) if (z[i] == key) return i;
        return -1;
    }
};

bool read_setfl(const std::string &path, HostPotential &p, std::string &err);
bool build_potential(int n_ele, const int32_t *zs, int nrho, double drho, int nr, double dr, double cutoff,
                     const double *F, const double *rho, const double *rphi, HostPotential &p, std::string &err);

// Offset tables (restatement of NeighbourIndex::make, src/atom/neighbour_index.inl:13-76) plus the
// real-space site vector (in units of a0) of every entry.
struct OffsetTable {
    std::vector<int64_t> off[2];          // full table per parity (0 even, 1 odd)
    std::vector<int64_t> half[2];
    std::vector<double> vec[2];           // 3 doubles per full entry
};
OffsetTable make_offsets(int64_t size_x, int64_t size_y, int cut_lattice, double rcf);

// Neighbour offset tables of one slot grid, passed to the kernels by value as a __grid_constant__
// parameter (13 KB, within the 32 KB parameter space): every context carries its own, and the
// candidate loops read them as warp-uniform constant-bank loads.
struct NeighTables {
    int nfull, npruned;
    int full[2][kMaxFull];      // reference order (inter-atom passes), linear slot offsets
    int lat[2][kMaxFull];       // gather order: entries within rc + 0.4 a0 first; linear offsets
    // gather order, mixed form: site_j - site_i in units of a0/2 (x, y, z; small exact integers) and
    // the parity-split index delta (w, as int bits): one 16-byte constant load per candidate
    float4 cand[2][kMaxFull];
};

// ---- kernel launchers (defined in the .cu files) ----
struct LaunchCtx {
    cudaStream_t stream;
    int num_sms;
    int rho_order = 0, rho_block = 256, rho_apt = 1;        // gather thread order, block size and atoms per thread
    int force_order = 0, force_block = 256, force_apt = 1;  // of the density and force passes (mg_autotune)
    const NeighTables *nt = nullptr;         // the context's offset tables
};

// Mass table shared by all contexts (atom types are fixed).
void set_mass_table(cudaStream_t stream);

// AoS <-> SoA over the slots [s0, s1) (s1 < 0: to the end of the grid)
void launch_unpack_aos(const LaunchCtx &lc, const Geom &g, const mg_atom_element *aos, Slots s, Inter in, int types_ok_mask,
                       bool mixed, int s0 = 0, int s1 = -1);
// set CNT_INTER = n_inter and clear the ghost and displaced counts
void launch_set_counts(const LaunchCtx &lc, Inter in, int n_inter);
void launch_pack_aos(const LaunchCtx &lc, const Geom &g, mg_atom_element *aos, Slots s, int fields, bool mixed,
                     int s0 = 0, int s1 = -1);
enum { PACK_ALL = 0xff, PACK_RHO = 1, PACK_DF = 2, PACK_F = 4 };

// local atoms [t0, t1) in k, j, i order (t1 < 0: all)
// fused: the previous force pass took this firststep already (launch_lat_force with fuse_next)
// alt: a body of a graph whose bodies alternate their u4 buffers (the previous body's records are in
// s.u4n)
void launch_firststep(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, const StepParams *sp, bool decide, int t0 = 0,
                      int t1 = -1, bool fused = false, bool alt = false);
// fill g.site_half (once per context)
void launch_site_table(const LaunchCtx &lc, const Geom &g, double *site_half);
void launch_decide_scan(const LaunchCtx &lc, const Geom &g, Slots s, Inter in);
// after a deciding firststep: the displaced slots in scan order into in.displaced, count in CNT_DISPLACED
void launch_displaced_collect(const LaunchCtx &lc, const Geom &g, Inter in);
// far-atom neighbourhood marks: clear those of the current far list / set them (grid-wide)
void launch_far_clear(const LaunchCtx &lc, const Geom &g, Inter in);
void launch_far_mark(const LaunchCtx &lc, const Geom &g, Inter in);
void launch_ghost_copy(const LaunchCtx &lc, const Geom &g, Slots s, bool mixed);
void launch_ghost_df(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, bool mixed);
// lists (mixed form): check or rebuild, per 32-site group, the list of pruned candidates that some site
// of the group has inside rc + skin, and visit only those (when lists_ok; the force pass of the same
// step must get the same flag)
void launch_lat_rho(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, bool hook,
                    bool lists = false);
// the density pass over the sites [u0, u1) of both parities (as launch_lat_force_sites)
void launch_lat_rho_sites(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, int u0, int u1,
                          bool lists = false);
bool lists_ok(const LaunchCtx &lc, const Geom &g);
// after the density pass of a step that used the group lists, before the next firststep: fold the
// step's maximum displacement into the skin's sum (or restart it when the pass rebuilt the words)
void launch_skin_advance(const LaunchCtx &lc, Slots s);
// a displacement record changed outside firststep: the next density pass rebuilds every group's list
void launch_skin_dirty(const LaunchCtx &lc, Slots s);
// forward df for the ghost slots inside local planes [k0, k1), or (k0 < 0) the ghost planes below and
// above the box plus the ghost inter atoms
void launch_ghost_df_planes(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, bool mixed, int k0, int k1);
// the lattice ghost copy for the ghost slots inside the local planes [k0, k1), or (k0 < 0) for the
// ghost planes below and above the box
void launch_ghost_copy_planes(const LaunchCtx &lc, const Geom &g, Slots s, int k0, int k1);
// The overlapped host step's decide on the local indices [t0, t1) after their firststep (no inter atoms
// in): a displaced atom nearest its own site goes into the list and back, leaving a new displacement
// record and a far-list entry whose neighbourhood is marked here; any other sets CNT_SPEC_VOID.
void launch_spec_decide(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, int t0, int t1);
// CNT_FAR = 0 and CNT_SPEC_VOID = 0 (after the previous far list's marks are cleared)
void launch_spec_begin(const LaunchCtx &lc, Inter in);
void launch_lat_df(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, bool hook);
// fuse_next (mixed form, kick, fixed dt): after the second half-kick each lattice atom also takes the
// next step's firststep (into u4n), when no inter atoms exist
void launch_lat_force(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, StepParams *sp, bool kick,
                      bool mixed, bool hook, bool fuse_next = false, bool lists = false);
// the force pass over the sites of both parities whose index within their parity is in [u0, u1):
// with u0 and u1 multiples of 32 (or u1 = n_local_half) the slabs of a split pass are disjoint warps
void launch_lat_force_sites(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, StepParams *sp, bool kick,
                            bool mixed, int u0, int u1, bool lists = false);
void launch_secondstep(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, StepParams *sp, bool lattice);
// step head: records the step's dt and, in variable mode, sets dt from the last kick's max |v|
void launch_step_head(const LaunchCtx &lc, StepParams *sp);
// out[0] = steps taken, out[1] = simulated time
void launch_clock_sample(const LaunchCtx &lc, const StepParams *sp, double *out);
// set the timestep rule and dt / dt/(2m) (dx_max <= 0: fixed dt)
void launch_set_step(const LaunchCtx &lc, StepParams *sp, double dt, double dx_max, double dt_min, double dt_max);
// recompute the max |v|^2 words from the state (after uploads, setv, rescale, single phases)
void launch_vmax_full(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, StepParams *sp);
void launch_energy(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed);
// far atoms: rebuild the list and its neighbourhood marks from positions (uploads, hooks)
void launch_far_rebuild(const LaunchCtx &lc, const Geom &g, Slots s, Inter in);
void launch_inter_manage(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, int steps_mask, bool mixed);
enum { MANAGE_DECIDE = 1, MANAGE_CLEAR_GHOST = 2, MANAGE_EXCHANGE = 4, MANAGE_BORDER = 8, MANAGE_INDEX = 16 };
void launch_inter_rho(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed);
// kick: the second half-kick of the lattice owners the density pass's inter-atom sweep listed (the
// lattice force pass kicked every other atom)
void launch_inter_force(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, StepParams *sp,
                        bool kick);
void launch_inter_energy(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed);
void launch_inter_firststep(const LaunchCtx &lc, Inter in, const StepParams *sp);
void launch_setv(const LaunchCtx &lc, const Geom &g, Slots s, int64_t slot, const double dir[3], double energy);
void launch_rescale(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, const double *d_factor_src, double t_set,
                    uint64_t n_atoms);
// thermo reduction: out[0] mvv, out[1..3] force sum, out[4] epot, out[5] vacancies
void launch_thermo(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, bool with_energy, double *partials,
                   int n_partials, double *out);
void launch_ws_map(const LaunchCtx &lc, const Geom &g, const double *xyz, int64_t n, int64_t *coords, uint32_t *flags,
                   int64_t *index);
// atom dump: the records of one frame (inter atoms in list order, then the box's lattice atoms in
// k, j, i order without vacancies) into out; *count = records. scratch: dump_scratch_ints(g) ints.
constexpr int kDumpThreads = 256;
inline int dump_scratch_ints(const Geom &g) { return (g.n_local + kDumpThreads - 1) / kDumpThreads; }
void launch_dump_pack(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, mg_dump_record *out,
                      unsigned long long *count, int *scratch, uint64_t step);

// mg_api.cpp services for the dump writer (mg_dump.cpp)
struct DumpSource {
    cudaStream_t stream;
    int64_t max_records;   // local slots + inter-atom capacity
    int scratch_ints;
};
DumpSource dump_source(const mg_context *ctx);
mg_status dump_pack(mg_context *ctx, mg_dump_record *out, unsigned long long *count, int *scratch, uint64_t step);
void dump_detach(mg_context *ctx, const mg_dump *d);  // mg_dump_close: the stage machine forgets d
void dump_note_error(mg_context *ctx, const std::string &why);  // mg_last_error(ctx) reports it

}  // namespace mg
