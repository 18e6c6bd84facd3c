// C ABI of libmisa_gb300.so: context lifetime, device state, potential upload, the per-step kernel
// sequence (captured once as a CUDA graph), the reference's per-phase hooks and the thermo reductions.
// The call order of one step follows simulation::simulate (src/simulation.cpp:164-194).

#include <algorithm>
#include <cmath>
#include <cstddef>
#include <cstdio>
#include <cstring>
#include <string>
#include <array>
#include <mutex>
#include <vector>

#include "mg_internal.h"

using namespace mg;

namespace {

thread_local std::string g_create_error;

constexpr int kNumTimers = 12;  // events per timed step; the kernels between consecutive events are:
const char *kTimerNames[kNumTimers - 1] = {"firststep",  // step head and firststep
                                           "inter_firststep",
                                           "inter_manage",  // displaced collection, far marks and the list manager
                                           "ghost_copy", "lat_rho", "inter_rho", "lat_df", "ghost_df", "lat_force",
                                           "inter_force", "secondstep"};

}  // namespace

namespace mg {
// message returned by mg_last_error(NULL) (entry points that take no context)
void set_global_error(const char *msg) { g_create_error = msg ? msg : ""; }
}  // namespace mg

struct mg_context {
    int device = 0;
    int precision = MG_PREC_FP64;
    Geom g{};
    Slots s{};
    Inter in{};
    PotTables pt{};
    bool pot_ready = false;
    HostPotential hp;               // the spline coefficients in use
    int types_ok_mask = 0;          // bit t set: the potential has the element of atom type t
    std::vector<void *> dev_allocs;
    void *pot_mem = nullptr;
    OffsetTable offs;
    std::vector<int> lat_order[2];  // reordered full table (pruned entries first), linear offsets
    NeighTables nt{};               // the tables as the kernels receive them
    int n_full = 0, n_pruned = 0;
    cudaStream_t stream = nullptr;
    int num_sms = 1;
    StepParams *d_sp = nullptr;     // device-resident step parameters and dt history
    double dt = 0.0;                // fixed timestep (ps)
    double dx_max = 0.0, dt_min = 0.0, dt_max = 0.0;  // variable timestep rule; dx_max <= 0: fixed
    bool vmax_stale = true;         // velocities changed outside a kick: recompute max |v| first
    bool prepared = false;
    std::string err;
    mg_atom_element *d_aos = nullptr;
    mg_atom_element *d_aos_in = nullptr;  // the overlapped host step's input, kept for a full rerun
    double *d_partials = nullptr;
    double *d_thermo = nullptr;
    double *d_samples = nullptr;    // stage-machine thermo samples (8 doubles each)
    int64_t n_samples_cap = 0;
    int n_partials = 0;
    double *d_ws_xyz = nullptr;
    int64_t *d_ws_coords = nullptr, *d_ws_index = nullptr;
    uint32_t *d_ws_flags = nullptr;
    int64_t ws_cap = 0;
    cudaGraphExec_t graph_exec = nullptr;
    // fused multi-step graph: fuse_steps loop bodies whose force passes (all but the last) take the
    // next firststep (mixed form, fixed dt); < 2: off
    int fuse_steps = 16;
    cudaGraphExec_t graph_multi = nullptr;
    float4 *u4_main = nullptr, *u4_alt = nullptr;  // s.u4 and s.u4n outside fused graphs
    bool alt_bodies = false;        // capturing bodies that alternate u4 buffers
    bool graph_stale = true;
    uint64_t gen = 1;               // bumped whenever captured graphs of this context go stale
    int graph_prec = -1;
    int launches_per_step = 0;
    bool timing = false;
    std::vector<cudaEvent_t> ev;       // kNumTimers + 1 events per timed step
    std::vector<double> timer_ms;      // accumulated per kernel
    int64_t timed_steps = 0;
    bool energy_valid = false;
    // mg_step_host pipeline: z-slab chunks (< 2: off), its copy streams and events
    int host_chunks = 16;
    cudaStream_t copy_in = nullptr, copy_out = nullptr;
    std::vector<cudaEvent_t> pipe_ev;
    // stage-machine dumps (mg_set_stage_output)
    mg_dump *stage_dump = nullptr;
    uint64_t stage_dump_interval = 0;
    std::string origin_path;

    // [precision][rho, force] = {thread order, block size, atoms per thread}
    int tune[2][2][3] = {{{0, 256, 1}, {0, 256, 1}}, {{0, 256, 1}, {0, 256, 1}}};
    LaunchCtx lc() const {
        LaunchCtx l{stream, num_sms};
        l.nt = &nt;
        l.rho_order = tune[precision][0][0];
        l.rho_block = tune[precision][0][1];
        l.rho_apt = tune[precision][0][2];
        l.force_order = tune[precision][1][0];
        l.force_block = tune[precision][1][1];
        l.force_apt = tune[precision][1][2];
        return l;
    }
    bool mixed() const { return precision == MG_PREC_MIXED; }
};

#define MG_CK(call)                                                                             \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            ctx->err = std::string(#call) + ": " + cudaGetErrorString(e_);                     \
            return MG_ERR_CUDA;                                                                 \
        }                                                                                       \
    } while (0)

namespace {

template <class T>
cudaError_t dalloc(mg_context *ctx, T **p, size_t n) {
    void *q = nullptr;
    cudaError_t e = cudaMalloc(&q, n * sizeof(T) + 16);
    if (e == cudaSuccess) {
        ctx->dev_allocs.push_back(q);
        *p = static_cast<T *>(q);
    }
    return e;
}

// Verlet skin of the group candidate lists (mixed form), Angstrom. The lists then hold about the
// sixth shell besides the 58 neighbours inside the cutoff; at 600 K and dt = 1 fs they last about 8
// steps (0.15 to 0.25 A measured within 0.3% of each other on 16M atoms, 0.2 the fastest).
constexpr double kDefaultSkin = 0.2;
void set_skin(Geom &g, double skin) {
    g.skin_h = static_cast<float>(skin * g.inv_h);
    const double r = (g.rc + skin) * g.inv_h;
    g.rcs2_h = skin > 0.0 ? static_cast<float>(r * r) : g.rc2_h;
}

int next_pow2(int n) {
    int p = 1;
    while (p < n) p <<= 1;
    return p;
}

mg_status check_launch(mg_context *ctx) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        ctx->err = std::string("kernel launch: ") + cudaGetErrorString(e);
        return MG_ERR_CUDA;
    }
    return MG_OK;
}

// NewtonMotion::setTimestepLength + preComputeDtInv2m (src/newton_motion.cpp:13-28), on the device
// record; dx_max > 0 switches to the variable rule, which the step head applies from the next step
void set_dt(mg_context *ctx, double dt, double dx_max = 0.0, double dt_min = 0.0, double dt_max = 0.0) {
    ctx->dt = dt;
    ctx->dx_max = dx_max;
    ctx->dt_min = dt_min;
    ctx->dt_max = dt_max;
    launch_set_step(ctx->lc(), ctx->d_sp, dt, dx_max, dt_min, dt_max);
}

// timer helpers (direct launches only)
struct Timer {
    mg_context *ctx;
    int64_t step;
    void mark(int k) {
        if (!ctx->timing) return;
        cudaEventRecord(ctx->ev[static_cast<size_t>(step) * (kNumTimers + 1) + k], ctx->stream);
    }
};

// ---- the kernel sequences ----
void seq_firststep(mg_context *ctx, bool decide, Timer *t, bool fused = false) {
    const LaunchCtx lc = ctx->lc();
    launch_firststep(lc, ctx->g, ctx->s, ctx->in, ctx->d_sp, decide, 0, -1, fused, ctx->alt_bodies);
    if (t) t->mark(1);
    launch_inter_firststep(lc, ctx->in, ctx->d_sp);
    if (t) t->mark(2);
}
// computeEam's list work (decide, exchangeInter, borderInter, makeIndex) and the lattice ghost copy
void seq_eam_lists(mg_context *ctx, bool with_manage_prefix, int manage_mask, Timer *t) {
    const LaunchCtx lc = ctx->lc();
    const bool mx = ctx->mixed();
    const bool decide = with_manage_prefix && (manage_mask & MANAGE_DECIDE);
    if (decide) {
        launch_displaced_collect(lc, ctx->g, ctx->in);  // the displaced slots of firststep, in scan order
        launch_far_clear(lc, ctx->g, ctx->in);           // the previous far list's neighbourhood marks
    }
    if (with_manage_prefix) launch_inter_manage(lc, ctx->g, ctx->s, ctx->in, manage_mask | MANAGE_INDEX, mx);
    else launch_inter_manage(lc, ctx->g, ctx->s, ctx->in, MANAGE_INDEX, mx);
    if (decide) launch_far_mark(lc, ctx->g, ctx->in);   // the new far list's neighbourhoods
    if (t) t->mark(3);
    launch_ghost_copy(lc, ctx->g, ctx->s, mx);
    if (t) t->mark(4);
}
// rho, dF/drho and the forward df exchange; the density pass checks or rebuilds the group lists that
// the force pass on the same positions walks
void seq_eam_rho(mg_context *ctx, Timer *t) {
    const LaunchCtx lc = ctx->lc();
    const bool mx = ctx->mixed();
    launch_lat_rho(lc, ctx->g, ctx->s, ctx->in, ctx->pt, mx, false, true);
    if (t) t->mark(5);
    launch_inter_rho(lc, ctx->g, ctx->s, ctx->in, ctx->pt, mx);
    if (t) t->mark(6);
    launch_lat_df(lc, ctx->g, ctx->s, ctx->in, ctx->pt, mx, false);
    if (t) t->mark(7);
    launch_ghost_df(lc, ctx->g, ctx->s, ctx->in, mx);
    if (t) t->mark(8);
}
// the inter-atom force pass and the second half-kick, after the lattice force pass
void seq_eam_force_tail(mg_context *ctx, bool kick, Timer *t) {
    const LaunchCtx lc = ctx->lc();
    launch_inter_force(lc, ctx->g, ctx->s, ctx->in, ctx->pt, ctx->mixed(), ctx->d_sp, kick);
    if (t) t->mark(10);
    if (kick) launch_secondstep(lc, ctx->g, ctx->s, ctx->in, ctx->d_sp, false);
    if (t) t->mark(11);
}
void seq_compute_eam(mg_context *ctx, bool kick, bool with_manage_prefix, int manage_mask, Timer *t, bool fuse_next = false) {
    seq_eam_lists(ctx, with_manage_prefix, manage_mask, t);
    seq_eam_rho(ctx, t);
    launch_lat_force(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, kick, ctx->mixed(), false, fuse_next, true);
    if (t) t->mark(9);
    seq_eam_force_tail(ctx, kick, t);
}
// one loop body: firststep, decide, exchangeInter, borderInter, exchangeAtom, computeEam, secondstep.
// fused_prev: the previous body's force pass took this firststep; fuse_next: this force pass takes the
// next one (both only act when no inter atoms exist, which the kernels check on the device)
void seq_step(mg_context *ctx, Timer *t, bool fused_prev = false, bool fuse_next = false) {
    if (t) t->mark(0);
    launch_step_head(ctx->lc(), ctx->d_sp);
    seq_firststep(ctx, true, t, fused_prev);
    seq_compute_eam(ctx, true, true, MANAGE_DECIDE | MANAGE_CLEAR_GHOST | MANAGE_EXCHANGE | MANAGE_BORDER, t, fuse_next);
}
// steps of mg_simulate that run fused: the mixed form with a fixed dt
bool fusable(const mg_context *ctx) { return ctx->fuse_steps >= 2 && ctx->mixed() && ctx->dx_max <= 0.0; }
constexpr int kLaunchesPerStep = 20;

mg_status require_ready(mg_context *ctx) {
    if (!ctx->pot_ready) { ctx->err = "potential not initialised"; return MG_ERR_POTENTIAL; }
    return MG_OK;
}

mg_status ensure_aos(mg_context *ctx) {
    if (ctx->d_aos) return MG_OK;
    MG_CK(dalloc(ctx, &ctx->d_aos, static_cast<size_t>(ctx->g.n_slots)));
    return MG_OK;
}

float int_bits_as_float(int i) {
    float f;
    std::memcpy(&f, &i, sizeof(f));
    return f;
}

mg_status upload_tables(mg_context *ctx) {
    const int n = ctx->n_full;
    NeighTables &nt = ctx->nt;
    std::memset(&nt, 0, sizeof(nt));
    nt.nfull = n;
    nt.npruned = ctx->n_pruned;
    // gather order (pruned entries first): linear offsets, parity-split index deltas, and the site
    // vectors in units of a0/2 (2 * the vector in units of a0: small exact integers)
    const int64_t half = ctx->g.half;
    for (int p = 0; p < 2; p++) {
        for (int q = 0; q < n; q++) {
            nt.full[p][q] = static_cast<int>(ctx->offs.off[p][q]);
            const int e = ctx->lat_order[p][q];
            const int64_t o = ctx->offs.off[p][e];
            nt.lat[p][q] = static_cast<int>(o);
            // slot s = 2k + p maps to p * half + k; its neighbour s + o has parity p2 and
            // (s + o) >> 1 = k + floor((p + o) / 2)
            const int64_t po = p + o;
            const int64_t p2 = ((po % 2) + 2) % 2;
            const int64_t fl = po >= 0 ? po / 2 : -((-po + 1) / 2);
            const int delta = static_cast<int>((p2 - p) * half + fl);
            const double *v = &ctx->offs.vec[p][3 * e];
            nt.cand[p][q] = make_float4((float) (2.0 * v[0]), (float) (2.0 * v[1]), (float) (2.0 * v[2]),
                                        int_bits_as_float(delta));
        }
    }
    set_mass_table(ctx->stream);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) { ctx->err = std::string("mass table: ") + cudaGetErrorString(e); return MG_ERR_CUDA; }
    return MG_OK;
}

mg_status install_potential(mg_context *ctx, const HostPotential &hp) {
    // Tables by atom type (3 x nr / nrho knots) and by type pair (9 x nr, ti * 3 + tj); types whose
    // element the file lacks point at element 0 and are rejected at upload (types_ok_mask).
    int ele_of_type[3];
    ctx->types_ok_mask = 0;
    for (int t = 0; t < 3; t++) {
        const int e = hp.ele(type_key(t));
        if (e >= 0) ctx->types_ok_mask |= 1 << t;
        ele_of_type[t] = e >= 0 ? e : 0;
    }
    if ((hp.nr - 1) * hp.dr + 1e-12 < ctx->g.rc) {  // the hit test uses rc = a0 * cutoff_radius_factor
        ctx->err = "potential r-table shorter than the cutoff radius";
        return MG_ERR_POTENTIAL;
    }
    const size_t nr = hp.nr, nrho = hp.nrho;
    const size_t n_rec = 3 * nr + 3 * nrho + 9 * nr;
    std::vector<Knot64> vd(n_rec), dd(n_rec);
    std::vector<float4> vf(n_rec), df(n_rec);
    size_t at = 0;
    auto put = [&](const HostSpline &sp) {
        for (int m = 0; m < sp.n; m++, at++) {
            vd[at] = Knot64{sp.c0[m], sp.c1[m], sp.c2[m], sp.c3[m]};
            dd[at] = Knot64{sp.d0[m], sp.d1[m], sp.d2[m], 0.0};
            vf[at] = make_float4((float) sp.c0[m], (float) sp.c1[m], (float) sp.c2[m], (float) sp.c3[m]);
            df[at] = make_float4((float) sp.d0[m], (float) sp.d1[m], (float) sp.d2[m], 0.0f);
        }
    };
    const size_t base_rho = 0, base_F = 3 * nr, base_z = 3 * nr + 3 * nrho;
    for (int t = 0; t < 3; t++) put(hp.rho[ele_of_type[t]]);
    for (int t = 0; t < 3; t++) put(hp.F[ele_of_type[t]]);
    for (int a = 0; a < 3; a++)
        for (int b = 0; b < 3; b++) put(hp.z2[HostPotential::pair_index(ele_of_type[a], ele_of_type[b])]);
    if (ctx->pot_mem) { cudaFree(ctx->pot_mem); ctx->pot_mem = nullptr; }
    // force records: pair (a, b) knot m = z c0..c3 of pair (a, b) and rho' d0..d2 of type b
    const size_t n_zr = 9 * nr;
    std::vector<float> zr(8 * n_zr, 0.0f);
    for (int a = 0; a < 3; a++) {
        for (int b = 0; b < 3; b++) {
            const HostSpline &z = hp.z2[HostPotential::pair_index(ele_of_type[a], ele_of_type[b])];
            const HostSpline &rb = hp.rho[ele_of_type[b]];
            for (size_t m = 0; m < nr; m++) {
                float *r = &zr[8 * ((a * 3 + b) * nr + m)];
                // interleaved for a packed Horner step: {c0, d0, c1, d1, c2, d2, c3, 0}
                r[0] = (float) z.c0[m]; r[1] = (float) rb.d0[m];
                r[2] = (float) z.c1[m]; r[3] = (float) rb.d1[m];
                r[4] = (float) z.c2[m]; r[5] = (float) rb.d2[m];
                r[6] = (float) z.c3[m]; r[7] = 0.0f;
            }
        }
    }
    const size_t bytes = n_rec * (2 * sizeof(Knot64) + 2 * sizeof(float4)) + zr.size() * sizeof(float);
    MG_CK(cudaMalloc(&ctx->pot_mem, bytes));
    Knot64 *d_vd = static_cast<Knot64 *>(ctx->pot_mem);
    Knot64 *d_dd = d_vd + n_rec;
    float4 *d_vf = reinterpret_cast<float4 *>(d_dd + n_rec);
    float4 *d_df = d_vf + n_rec;
    float *d_zr = reinterpret_cast<float *>(d_df + n_rec);  // 32-byte aligned: every block above is a multiple of 32 bytes
    MG_CK(cudaMemcpy(d_vd, vd.data(), n_rec * sizeof(Knot64), cudaMemcpyHostToDevice));
    MG_CK(cudaMemcpy(d_dd, dd.data(), n_rec * sizeof(Knot64), cudaMemcpyHostToDevice));
    MG_CK(cudaMemcpy(d_vf, vf.data(), n_rec * sizeof(float4), cudaMemcpyHostToDevice));
    MG_CK(cudaMemcpy(d_df, df.data(), n_rec * sizeof(float4), cudaMemcpyHostToDevice));
    MG_CK(cudaMemcpy(d_zr, zr.data(), zr.size() * sizeof(float), cudaMemcpyHostToDevice));

    PotTables &pt = ctx->pt;
    pt.nr = hp.nr;
    pt.nrho = hp.nrho;
    pt.inv_dr = hp.rho[0].inv_delta;
    pt.inv_drho = hp.F[0].inv_delta;
    pt.inv_dr_f = (float) pt.inv_dr;
    pt.inv_drho_f = (float) pt.inv_drho;
    pt.h_inv_dr_f = (float) (0.5 * ctx->g.a0 * pt.inv_dr);
    pt.rho_v = d_vd + base_rho; pt.rho_d = d_dd + base_rho;
    pt.F_v = d_vd + base_F; pt.F_d = d_dd + base_F;
    pt.z_v = d_vd + base_z; pt.z_d = d_dd + base_z;
    pt.rho_vf = d_vf + base_rho; pt.rho_dff = d_df + base_rho;
    pt.F_vf = d_vf + base_F; pt.F_dff = d_df + base_F;
    pt.z_vf = d_vf + base_z; pt.z_dff = d_df + base_z;
    pt.zr8 = d_zr;
    ctx->hp = hp;
    ctx->pot_ready = true;
    ctx->graph_stale = true;
    ctx->gen++;  // rebuild graphs
    return MG_OK;
}

mg_status check_types(mg_context *ctx, const mg_atom_element *atoms, int64_t n) {
    for (int64_t i = 0; i < n; i++) {
        const int t = atoms[i].type;
        if (t < -1 || t > 2) { ctx->err = "atom type out of range"; return MG_ERR_ARG; }
        if (t >= 0 && !(ctx->types_ok_mask & (1 << t))) { ctx->err = "potential has no element for an atom type present"; return MG_ERR_POTENTIAL; }
    }
    return MG_OK;
}

mg_status build_graph(mg_context *ctx) {
    if (ctx->graph_exec && !ctx->graph_stale && ctx->graph_prec == ctx->precision) return MG_OK;
    if (ctx->graph_exec) { cudaGraphExecDestroy(ctx->graph_exec); ctx->graph_exec = nullptr; }
    if (ctx->graph_multi) { cudaGraphExecDestroy(ctx->graph_multi); ctx->graph_multi = nullptr; }
    cudaGraph_t graph;
    MG_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    seq_step(ctx, nullptr);
    MG_CK(cudaStreamEndCapture(ctx->stream, &graph));
    size_t n_nodes = 0;
    cudaGraphGetNodes(graph, nullptr, &n_nodes);
    ctx->launches_per_step = static_cast<int>(n_nodes);
    cudaError_t e = cudaGraphInstantiate(&ctx->graph_exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { ctx->err = std::string("graph instantiate: ") + cudaGetErrorString(e); return MG_ERR_CUDA; }
    ctx->graph_stale = false;
    ctx->graph_prec = ctx->precision;
    return MG_OK;
}

// The u4 buffers of body i of k fused bodies: its own and the next body's alternate, and the last
// body's own is the context's usual one, so between launches u4 is where every other call expects it.
void set_body_buffers(mg_context *ctx, int64_t k, int64_t i) {
    const bool own_is_main = ((k - 1 - i) % 2) == 0;
    ctx->s.u4 = own_is_main ? ctx->u4_main : ctx->u4_alt;
    ctx->s.u4n = own_is_main ? ctx->u4_alt : ctx->u4_main;
}

// fuse_steps loop bodies in one graph: the first takes its own firststep, the last does not take the
// next one, so the state between launches is the end of a loop body as always
mg_status build_graph_multi(mg_context *ctx) {
    mg_status st = build_graph(ctx);
    if (st != MG_OK || ctx->graph_multi) return st;
    cudaGraph_t graph;
    MG_CK(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    const int k = ctx->fuse_steps;
    ctx->alt_bodies = true;
    for (int i = 0; i < k; i++) {
        set_body_buffers(ctx, k, i);
        seq_step(ctx, nullptr, i > 0, i < k - 1);
    }
    ctx->alt_bodies = false;
    set_body_buffers(ctx, k, k - 1);
    MG_CK(cudaStreamEndCapture(ctx->stream, &graph));
    cudaError_t e = cudaGraphInstantiate(&ctx->graph_multi, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { ctx->err = std::string("graph instantiate: ") + cudaGetErrorString(e); return MG_ERR_CUDA; }
    return MG_OK;
}

mg_status read_device_errors(mg_context *ctx, uint32_t *bits) {
    int cnt[CNT_WORDS];
    MG_CK(cudaMemcpyAsync(cnt, ctx->in.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    *bits = static_cast<uint32_t>(cnt[CNT_ERRORS]);
    return MG_OK;
}

mg_status status_from_bits(mg_context *ctx, uint32_t bits) {
    if (bits & MG_DEVERR_BAD_TYPE) { ctx->err = "atom type out of range or without a potential element"; return MG_ERR_ARG; }
    if (bits & MG_DEVERR_OUT_OF_GRID) { ctx->err = "an index left the slot grid"; return MG_ERR_OUT_OF_GRID; }
    if (bits & (MG_DEVERR_INTER_OVERFLOW | MG_DEVERR_GHOST_OVERFLOW | MG_DEVERR_DISPLACED_OVERFLOW)) {
        ctx->err = "inter-atom list capacity exceeded";
        return MG_ERR_CAPACITY;
    }
    return MG_OK;
}

}  // namespace

extern "C" {

mg_status mg_env_init(int32_t device) {
    cudaError_t e = cudaSetDevice(device);
    if (e != cudaSuccess) { g_create_error = cudaGetErrorString(e); return MG_ERR_CUDA; }
    return MG_OK;
}
mg_status mg_env_clean(void) { return MG_OK; }

const char *mg_last_error(const mg_context *ctx) { return ctx ? ctx->err.c_str() : g_create_error.c_str(); }

mg_status mg_create(const int64_t phase_space[3], double lattice_const, double rcf, int32_t precision,
                    int64_t inter_capacity, mg_context **out) {
    if (!out || !phase_space || !(lattice_const > 0) || !(rcf > 0)) { g_create_error = "bad argument"; return MG_ERR_ARG; }
    if (precision != MG_PREC_FP64 && precision != MG_PREC_MIXED) { g_create_error = "bad precision"; return MG_ERR_ARG; }
    *out = nullptr;
    const int ghost = static_cast<int>(std::ceil(rcf)) + 1;       // src/simulation.cpp:46
    const int cut_lattice = static_cast<int>(std::ceil(rcf));      // libcomm cut_lattice
    for (int d = 0; d < 3; d++) {
        if (phase_space[d] < 2 * ghost) { g_create_error = "every dimension needs at least 2*ghost unit cells"; return MG_ERR_ARG; }
        if (phase_space[d] > (1 << 20)) { g_create_error = "box too large for 32-bit slot indices"; return MG_ERR_ARG; }
    }
    const int64_t Sx = 2 * (phase_space[0] + 2 * ghost), Sy = phase_space[1] + 2 * ghost, Sz = phase_space[2] + 2 * ghost;
    if (Sx * Sy * Sz >= (int64_t) 0x7fffffff - 1024) { g_create_error = "box too large for 32-bit slot indices"; return MG_ERR_ARG; }

    auto *ctx = new mg_context();
    ctx->precision = precision;
    cudaGetDevice(&ctx->device);
    Geom &g = ctx->g;
    g.Sx = (int) Sx; g.Sy = (int) Sy; g.Sz = (int) Sz;
    g.gx = 2 * ghost; g.gy = ghost; g.gz = ghost;
    g.bx = (int) (2 * phase_space[0]); g.by = (int) phase_space[1]; g.bz = (int) phase_space[2];
    g.n_slots = (int) (Sx * Sy * Sz);
    g.n_local = g.bx * g.by * g.bz;
    g.n_ghost_slots = g.n_slots - g.n_local;
    g.half = g.n_slots / 2;  // Sx is even, so slot parity is x parity
    g.nxh = g.bx / 2;
    g.n_local_half = g.n_local / 2;
    for (int d = 0; d < 3; d++) g.cells[d] = (int) phase_space[d];
    g.a0 = lattice_const;
    g.rc = lattice_const * rcf;  // atom::atom, src/atom.cpp:14-19
    g.rc2 = g.rc * g.rc;
    g.thr = std::pow(0.2 * lattice_const, 2.0);
    for (int d = 0; d < 3; d++) g.L[d] = phase_space[d] * lattice_const;
    g.inv_h = 2.0 / lattice_const;
    g.inv_a0 = 1.0 / lattice_const;
    g.h_f = (float) (0.5 * lattice_const);
    g.inv_h_f = (float) g.inv_h;
    g.thr_lo_f = (float) (g.thr * (1.0 - 1e-4));
    g.rc2_h = (float) (g.rc2 * g.inv_h * g.inv_h);
    g.rc2_pre = (float) ((double) g.rc2_h * (1.0 + 1e-4));
    set_skin(g, kDefaultSkin);

    // offset tables, and the lattice gather order: pruned entries (site distance below
    // rc + 0.4 a0, with margin) first, in reference order, then the rest
    ctx->offs = make_offsets(Sx, Sy, cut_lattice, rcf);
    ctx->n_full = static_cast<int>(ctx->offs.off[0].size());
    if (ctx->n_full > kMaxFull || ctx->offs.off[1].size() != ctx->offs.off[0].size()) {
        g_create_error = "offset table too large";
        delete ctx;
        return MG_ERR_ARG;
    }
    // The pruned entries keep the reference order, which is also memory order (sorting them by site
    // distance scattered the neighbour loads: +6% per pass).
    const double prune_r = rcf + 0.4 + 1e-6;
    for (int p = 0; p < 2; p++) {
        std::vector<int> near, rest;
        for (int q = 0; q < ctx->n_full; q++) {
            const double *v = &ctx->offs.vec[p][3 * q];
            const double r = std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]);
            (r < prune_r ? near : rest).push_back(q);
        }
        if (p == 0) ctx->n_pruned = static_cast<int>(near.size());
        ctx->lat_order[p] = near;
        ctx->lat_order[p].insert(ctx->lat_order[p].end(), rest.begin(), rest.end());
    }

    cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) { g_create_error = cudaGetErrorString(e); delete ctx; return MG_ERR_CUDA; }
    cudaDeviceGetAttribute(&ctx->num_sms, cudaDevAttrMultiProcessorCount, ctx->device);

    auto fail = [&](cudaError_t err) {
        g_create_error = std::string("device allocation: ") + cudaGetErrorString(err);
        mg_destroy(ctx);
        return MG_ERR_CUDA;
    };
    const size_t ns = static_cast<size_t>(g.n_slots);
    Slots &s = ctx->s;
    cudaError_t ae = cudaSuccess;
#define ALLOC(p, n) do { if ((ae = dalloc(ctx, &(p), (n))) != cudaSuccess) return fail(ae); } while (0)
    ALLOC(s.x, ns); ALLOC(s.y, ns); ALLOC(s.z, ns);
    ALLOC(s.vx, ns); ALLOC(s.vy, ns); ALLOC(s.vz, ns);
    ALLOC(s.fx, ns); ALLOC(s.fy, ns); ALLOC(s.fz, ns);
    ALLOC(s.rho, ns); ALLOC(s.df, ns); ALLOC(s.e, ns);
    ALLOC(s.type, ns); ALLOC(s.id, ns);
    ALLOC(s.u4, ns); ALLOC(s.u4n, ns); ALLOC(s.df32, ns);
    ALLOC(s.near, static_cast<size_t>(2 * kListWords * ((g.n_local_half + 31) / 32)));
    ALLOC(s.skin, 1);
    ctx->u4_main = s.u4;
    ctx->u4_alt = s.u4n;

    Inter &in = ctx->in;
    in.cap = static_cast<int>(inter_capacity > 0 ? inter_capacity : 16384);
    in.gcap = 8 * in.cap;
    in.dcap = next_pow2(in.cap);
    in.fcap = in.cap;
    const int nbuck = next_pow2(std::max(in.cap + in.gcap, in.dcap));
    const size_t cap = in.cap, gcap = in.gcap;
    ALLOC(in.cnt, CNT_WORDS);
    ALLOC(in.id, cap); ALLOC(in.type, cap);
    ALLOC(in.x, cap); ALLOC(in.y, cap); ALLOC(in.z, cap);
    ALLOC(in.vx, cap); ALLOC(in.vy, cap); ALLOC(in.vz, cap);
    ALLOC(in.fx, cap); ALLOC(in.fy, cap); ALLOC(in.fz, cap);
    ALLOC(in.rho, cap); ALLOC(in.df, cap); ALLOC(in.e, cap);
    ALLOC(in.gtype, gcap); ALLOC(in.groot, gcap);
    ALLOC(in.gx, gcap); ALLOC(in.gy, gcap); ALLOC(in.gz, gcap); ALLOC(in.gdf, gcap);
    ALLOC(in.scratch_i, 3 * cap); ALLOC(in.scratch_d, 13 * cap); ALLOC(in.scratch_u, cap);
    ALLOC(in.displaced, (size_t) in.dcap);
    {
        const size_t nblocks = (static_cast<size_t>(g.n_local) + kFirstThreads - 1) / kFirstThreads;
        ALLOC(in.dflag, nblocks * kFirstThreads);
        ALLOC(in.dblock, nblocks);
    }
    ALLOC(in.claim, ns);
    ALLOC(in.far_list, (size_t) in.fcap);
    ALLOC(in.far_flag, ns);
    ALLOC(in.bucket, (size_t) nbuck);
    ALLOC(in.n_bucket, 1);
    // every local inter atom lists at most its nearest site and the full offsets of that site
    in.tcap = static_cast<int>(std::min<int64_t>(g.n_local, static_cast<int64_t>(in.cap) * (kMaxFull + 1)));
    ALLOC(in.touch_bits, ns / 32 + 1);
    ALLOC(in.touched, (size_t) in.tcap);
    ctx->n_partials = ctx->num_sms * 4;
    ALLOC(ctx->d_partials, (size_t) ctx->n_partials * 8);
    ALLOC(ctx->d_thermo, 8);
    ALLOC(ctx->d_sp, 1);
    {
        double *site_half = nullptr;
        ctx->g.n_site_half = std::max(g.bx, std::max(2 * g.by, 2 * g.bz)) + 2;
        ALLOC(site_half, (size_t) ctx->g.n_site_half);
        ctx->g.site_half = site_half;
    }
#undef ALLOC
    e = cudaMemsetAsync(in.cnt, 0, CNT_WORDS * sizeof(int), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(in.claim, 0x7f, ns * sizeof(int), ctx->stream);  // 0x7f7f7f7f > any list index
    if (e == cudaSuccess) e = cudaMemsetAsync(in.far_flag, 0, ns, ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(in.n_bucket, 0, sizeof(int), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(in.touch_bits, 0, (ns / 32 + 1) * sizeof(unsigned), ctx->stream);
    if (e == cudaSuccess)  // the padding past n_local is never written and must read as "not displaced"
        e = cudaMemsetAsync(in.dflag, 0, ((static_cast<size_t>(g.n_local) + kFirstThreads - 1) / kFirstThreads) * kFirstThreads,
                            ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.type, 0xff, ns, ctx->stream);  // all slots INVALID
    if (e == cudaSuccess) e = cudaMemsetAsync(s.u4, 0xff, ns * sizeof(float4), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.u4n, 0xff, ns * sizeof(float4), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(ctx->d_sp, 0, sizeof(StepParams), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s.skin, 0, sizeof(SkinState), ctx->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(&s.skin->dirty, 1, 1, ctx->stream);
    if (e != cudaSuccess) return fail(e);
    if (upload_tables(ctx) != MG_OK) { g_create_error = ctx->err; mg_destroy(ctx); return MG_ERR_CUDA; }
    launch_site_table(ctx->lc(), ctx->g, const_cast<double *>(ctx->g.site_half));
    set_dt(ctx, 0.001);
    *out = ctx;
    return MG_OK;
}

mg_status mg_destroy(mg_context *ctx) {
    if (!ctx) return MG_ERR_ARG;
    if (ctx->stream) cudaStreamSynchronize(ctx->stream);
    if (ctx->graph_exec) cudaGraphExecDestroy(ctx->graph_exec);
    if (ctx->graph_multi) cudaGraphExecDestroy(ctx->graph_multi);
    for (cudaEvent_t e : ctx->ev) cudaEventDestroy(e);
    for (cudaEvent_t e : ctx->pipe_ev) cudaEventDestroy(e);
    if (ctx->copy_in) cudaStreamDestroy(ctx->copy_in);
    if (ctx->copy_out) cudaStreamDestroy(ctx->copy_out);
    for (void *p : ctx->dev_allocs) cudaFree(p);
    if (ctx->pot_mem) cudaFree(ctx->pot_mem);
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    delete ctx;
    return MG_OK;
}

mg_status mg_grid(const mg_context *ctx, int64_t out[6]) {
    if (!ctx || !out) return MG_ERR_ARG;
    out[0] = ctx->g.Sx; out[1] = ctx->g.Sy; out[2] = ctx->g.Sz;
    out[3] = ctx->g.gx; out[4] = ctx->g.gy; out[5] = ctx->g.gz;
    return MG_OK;
}

mg_status mg_set_precision(mg_context *ctx, int32_t precision) {
    if (!ctx || (precision != MG_PREC_FP64 && precision != MG_PREC_MIXED)) return MG_ERR_ARG;
    ctx->precision = precision;
    ctx->prepared = false;  // derived arrays (u4, df32) must be rebuilt by an upload
    ctx->gen++;
    return MG_OK;
}

mg_status mg_nei_offset_init(mg_context *ctx, const int64_t *full_even, const int64_t *full_odd, int32_t n_full,
                             const int64_t *half_even, const int64_t *half_odd, int32_t n_half) {
    if (!ctx || !full_even || !full_odd || !half_even || !half_odd) return MG_ERR_ARG;
    if (n_full != ctx->n_full || n_half != (int32_t) ctx->offs.half[0].size()) {
        ctx->err = "offset tables differ in length";
        return MG_ERR_ARG;
    }
    for (int i = 0; i < n_full; i++)
        if (full_even[i] != ctx->offs.off[0][i] || full_odd[i] != ctx->offs.off[1][i]) { ctx->err = "full offset tables differ"; return MG_ERR_ARG; }
    for (int i = 0; i < n_half; i++)
        if (half_even[i] != ctx->offs.half[0][i] || half_odd[i] != ctx->offs.half[1][i]) { ctx->err = "half offset tables differ"; return MG_ERR_ARG; }
    return MG_OK;
}

mg_status mg_nei_offsets(const mg_context *ctx, int32_t which, int64_t *out, int32_t cap, int32_t *n) {
    if (!ctx || !n || which < 0 || which > 5) return MG_ERR_ARG;
    std::vector<int64_t> v;
    if (which <= 1) v = ctx->offs.off[which];
    else if (which <= 3) v = ctx->offs.half[which - 2];
    else {
        const int p = which - 4;
        for (int q = 0; q < ctx->n_pruned; q++) v.push_back(ctx->offs.off[p][ctx->lat_order[p][q]]);
    }
    *n = static_cast<int32_t>(v.size());
    for (int32_t i = 0; i < *n && i < cap && out; i++) out[i] = v[i];
    return MG_OK;
}

mg_status mg_pot_init_setfl(mg_context *ctx, const char *path) {
    if (!ctx || !path) return MG_ERR_ARG;
    HostPotential hp;
    if (!read_setfl(path, hp, ctx->err)) return MG_ERR_POTENTIAL;
    return install_potential(ctx, hp);
}

mg_status mg_pot_init_tables(mg_context *ctx, int32_t n_ele, const int32_t *zs, int32_t nrho, double drho, int32_t nr,
                             double dr, double cutoff, const double *F, const double *rho, const double *rphi) {
    if (!ctx || !zs || !F || !rho || !rphi) return MG_ERR_ARG;
    HostPotential hp;
    if (!build_potential(n_ele, zs, nrho, drho, nr, dr, cutoff, F, rho, rphi, hp, ctx->err)) return MG_ERR_POTENTIAL;
    return install_potential(ctx, hp);
}

mg_status mg_pot_spline(const mg_context *ctx, int32_t kind, int32_t e1, int32_t e2, double *out, int32_t cap,
                        int32_t *n) {
    if (!ctx || !n || kind < 0 || kind > 2) return MG_ERR_ARG;
    if (!ctx->pot_ready) return MG_ERR_POTENTIAL;
    const HostPotential &p = ctx->hp;
    if (e1 < 0 || e1 >= p.n_ele || e2 < 0 || e2 >= p.n_ele) return MG_ERR_ARG;
    const HostSpline &sp = kind == 0 ? p.F[e1] : kind == 1 ? p.rho[e1] : p.z2[HostPotential::pair_index(e1, e2)];
    *n = sp.n;
    for (int m = 0; m < sp.n && out && 7 * m + 6 < cap; m++) {
        out[7 * m + 0] = sp.c0[m]; out[7 * m + 1] = sp.c1[m]; out[7 * m + 2] = sp.c2[m]; out[7 * m + 3] = sp.c3[m];
        out[7 * m + 4] = sp.d0[m]; out[7 * m + 5] = sp.d1[m]; out[7 * m + 6] = sp.d2[m];
    }
    return MG_OK;
}

// ---------------------------------------------------------------------------------------------
// hooks (src/arch/arch_imp.h:27-31)
// ---------------------------------------------------------------------------------------------
static mg_status hook_upload(mg_context *ctx, mg_atom_element *atoms, double cutoff) {
    if (!ctx || !atoms) return MG_ERR_ARG;
    mg_status st = require_ready(ctx);
    if (st != MG_OK) return st;
    if (std::fabs(cutoff - ctx->g.rc) > 1e-12 * ctx->g.rc) { ctx->err = "cutoff radius differs from the context's"; return MG_ERR_ARG; }
    if ((st = ensure_aos(ctx)) != MG_OK) return st;
    MG_CK(cudaMemcpyAsync(ctx->d_aos, atoms, sizeof(mg_atom_element) * ctx->g.n_slots, cudaMemcpyHostToDevice, ctx->stream));
    launch_unpack_aos(ctx->lc(), ctx->g, ctx->d_aos, ctx->s, ctx->in, ctx->types_ok_mask, ctx->mixed());
    launch_far_rebuild(ctx->lc(), ctx->g, ctx->s, ctx->in);
    ctx->vmax_stale = true;
    return check_launch(ctx);
}
static mg_status hook_download(mg_context *ctx, mg_atom_element *atoms, int fields) {
    launch_pack_aos(ctx->lc(), ctx->g, ctx->d_aos, ctx->s, fields, ctx->mixed());
    mg_status st = check_launch(ctx);
    if (st != MG_OK) return st;
    MG_CK(cudaMemcpyAsync(atoms, ctx->d_aos, sizeof(mg_atom_element) * ctx->g.n_slots, cudaMemcpyDeviceToHost, ctx->stream));
    uint32_t bits = 0;
    if ((st = read_device_errors(ctx, &bits)) != MG_OK) return st;
    return status_from_bits(ctx, bits);
}

mg_status mg_eam_rho_calc(mg_context *ctx, mg_atom_element *atoms, double cutoff_radius) {
    mg_status st = hook_upload(ctx, atoms, cutoff_radius);
    if (st != MG_OK) return st;
    launch_lat_rho(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->pt, ctx->mixed(), true);
    return hook_download(ctx, atoms, PACK_RHO);
}
mg_status mg_eam_df_calc(mg_context *ctx, mg_atom_element *atoms, double cutoff_radius) {
    mg_status st = hook_upload(ctx, atoms, cutoff_radius);
    if (st != MG_OK) return st;
    launch_lat_df(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->pt, ctx->mixed(), true);
    return hook_download(ctx, atoms, PACK_DF);
}
mg_status mg_eam_force_calc(mg_context *ctx, mg_atom_element *atoms, double cutoff_radius) {
    mg_status st = hook_upload(ctx, atoms, cutoff_radius);
    if (st != MG_OK) return st;
    launch_lat_force(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, false, ctx->mixed(), true);
    return hook_download(ctx, atoms, PACK_F);
}

// ---------------------------------------------------------------------------------------------
// resident state
// ---------------------------------------------------------------------------------------------
mg_status mg_upload(mg_context *ctx, const mg_atom_element *atoms, int64_t n_slots, const mg_atom_element *inter,
                    int64_t n_inter) {
    if (!ctx || !atoms || n_slots != ctx->g.n_slots || n_inter < 0 || (n_inter > 0 && !inter)) return MG_ERR_ARG;
    mg_status st = require_ready(ctx);
    if (st != MG_OK) return st;
    if (n_inter > ctx->in.cap) { ctx->err = "inter list larger than the context capacity"; return MG_ERR_CAPACITY; }
    if ((st = check_types(ctx, inter, n_inter)) != MG_OK) return st;
    if ((st = ensure_aos(ctx)) != MG_OK) return st;
    MG_CK(cudaMemcpyAsync(ctx->d_aos, atoms, sizeof(mg_atom_element) * n_slots, cudaMemcpyHostToDevice, ctx->stream));
    launch_unpack_aos(ctx->lc(), ctx->g, ctx->d_aos, ctx->s, ctx->in, ctx->types_ok_mask, ctx->mixed());
    // inter list: records -> SoA columns via host staging
    std::vector<uint64_t> id(n_inter);
    std::vector<int> ty(n_inter);
    std::vector<double> col(13 * (size_t) n_inter);
    for (int64_t a = 0; a < n_inter; a++) {
        const mg_atom_element &r = inter[a];
        id[a] = r.id; ty[a] = r.type;
        const double v[11] = {r.x[0], r.x[1], r.x[2], r.v[0], r.v[1], r.v[2], r.f[0], r.f[1], r.f[2], r.rho, r.df};
        for (int k = 0; k < 11; k++) col[k * n_inter + a] = v[k];
    }
    Inter &in = ctx->in;
    double *dst[11] = {in.x, in.y, in.z, in.vx, in.vy, in.vz, in.fx, in.fy, in.fz, in.rho, in.df};
    if (n_inter > 0) {
        MG_CK(cudaMemcpyAsync(in.id, id.data(), n_inter * sizeof(uint64_t), cudaMemcpyHostToDevice, ctx->stream));
        MG_CK(cudaMemcpyAsync(in.type, ty.data(), n_inter * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
        for (int k = 0; k < 11; k++)
            MG_CK(cudaMemcpyAsync(dst[k], col.data() + k * n_inter, n_inter * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    }
    // the ghost list and the displaced list restart empty; the far list is rebuilt from positions
    launch_set_counts(ctx->lc(), ctx->in, static_cast<int>(n_inter));
    launch_far_rebuild(ctx->lc(), ctx->g, ctx->s, ctx->in);
    ctx->prepared = false;
    ctx->vmax_stale = true;
    ctx->energy_valid = false;
    return check_launch(ctx);
}

mg_status mg_download(mg_context *ctx, mg_atom_element *atoms, int64_t n_slots, mg_atom_element *inter,
                      int64_t inter_cap, int64_t *n_inter) {
    if (!ctx || !atoms || n_slots != ctx->g.n_slots) return MG_ERR_ARG;
    mg_status st = ensure_aos(ctx);
    if (st != MG_OK) return st;
    launch_pack_aos(ctx->lc(), ctx->g, ctx->d_aos, ctx->s, PACK_ALL, ctx->mixed());
    if ((st = check_launch(ctx)) != MG_OK) return st;
    MG_CK(cudaMemcpyAsync(atoms, ctx->d_aos, sizeof(mg_atom_element) * n_slots, cudaMemcpyDeviceToHost, ctx->stream));
    int cnt[CNT_WORDS];
    MG_CK(cudaMemcpyAsync(cnt, ctx->in.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    const int64_t n = cnt[CNT_INTER];
    if (n_inter) *n_inter = n;
    const int64_t m = std::min<int64_t>(n, inter ? inter_cap : 0);
    if (m > 0) {
        Inter &in = ctx->in;
        std::vector<uint64_t> id(m);
        std::vector<int> ty(m);
        std::vector<double> col(11 * (size_t) m);
        const double *src[11] = {in.x, in.y, in.z, in.vx, in.vy, in.vz, in.fx, in.fy, in.fz, in.rho, in.df};
        MG_CK(cudaMemcpyAsync(id.data(), in.id, m * sizeof(uint64_t), cudaMemcpyDeviceToHost, ctx->stream));
        MG_CK(cudaMemcpyAsync(ty.data(), in.type, m * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        for (int k = 0; k < 11; k++)
            MG_CK(cudaMemcpyAsync(col.data() + k * m, src[k], m * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        MG_CK(cudaStreamSynchronize(ctx->stream));
        for (int64_t a = 0; a < m; a++) {
            mg_atom_element &r = inter[a];
            std::memset(&r, 0, sizeof(r));
            r.id = id[a]; r.type = ty[a];
            r.x[0] = col[0 * m + a]; r.x[1] = col[1 * m + a]; r.x[2] = col[2 * m + a];
            r.v[0] = col[3 * m + a]; r.v[1] = col[4 * m + a]; r.v[2] = col[5 * m + a];
            r.f[0] = col[6 * m + a]; r.f[1] = col[7 * m + a]; r.f[2] = col[8 * m + a];
            r.rho = col[9 * m + a]; r.df = col[10 * m + a];
        }
    }
    return MG_OK;
}

mg_status mg_download_ghost_inter(mg_context *ctx, mg_atom_element *ghost, int64_t cap, int64_t *n_ghost) {
    if (!ctx) return MG_ERR_ARG;
    int cnt[CNT_WORDS];
    MG_CK(cudaMemcpyAsync(cnt, ctx->in.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    const int64_t n = cnt[CNT_GHOST];
    if (n_ghost) *n_ghost = n;
    const int64_t m = std::min<int64_t>(n, ghost ? cap : 0);
    if (m > 0) {
        Inter &in = ctx->in;
        std::vector<int> ty(m);
        std::vector<double> col(4 * (size_t) m);
        const double *src[4] = {in.gx, in.gy, in.gz, in.gdf};
        MG_CK(cudaMemcpyAsync(ty.data(), in.gtype, m * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
        for (int k = 0; k < 4; k++)
            MG_CK(cudaMemcpyAsync(col.data() + k * m, src[k], m * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        MG_CK(cudaStreamSynchronize(ctx->stream));
        for (int64_t a = 0; a < m; a++) {
            mg_atom_element &r = ghost[a];
            std::memset(&r, 0, sizeof(r));
            r.type = ty[a];
            r.x[0] = col[a]; r.x[1] = col[m + a]; r.x[2] = col[2 * m + a];
            r.df = col[3 * m + a];
        }
    }
    return MG_OK;
}

mg_status mg_set_timestep(mg_context *ctx, double dt) {
    if (!ctx || !(dt > 0)) return MG_ERR_ARG;
    set_dt(ctx, dt);
    return check_launch(ctx);
}

mg_status mg_set_variable_timestep(mg_context *ctx, double dx_max, double dt_min, double dt_max) {
    if (!ctx) return MG_ERR_ARG;
    if (!(dx_max > 0) || !(dt_min > 0) || !(dt_max >= dt_min) || !std::isfinite(dt_max) || !std::isfinite(dx_max)) {
        ctx->err = "variable timestep needs dx_max > 0 and 0 < dt_min <= dt_max (finite)";
        return MG_ERR_ARG;
    }
    set_dt(ctx, dt_max, dx_max, dt_min, dt_max);
    ctx->vmax_stale = true;  // the fixed-dt kicks before this did not keep the max-|v| words
    return check_launch(ctx);
}

mg_status mg_clock(mg_context *ctx, int64_t *steps, double *time_ps, double *dt_ps) {
    if (!ctx) return MG_ERR_ARG;
    StepParams head;
    MG_CK(cudaMemcpyAsync(&head, ctx->d_sp, offsetof(StepParams, vmax2), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    if (steps) *steps = head.steps;
    if (time_ps) *time_ps = head.time;
    if (dt_ps) *dt_ps = head.dt;
    return MG_OK;
}

mg_status mg_dt_history(mg_context *ctx, double *out, int64_t cap, int64_t *n_out) {
    if (!ctx || cap < 0 || (cap > 0 && !out) || !n_out) return MG_ERR_ARG;
    int64_t steps = 0;
    mg_status st = mg_clock(ctx, &steps, nullptr, nullptr);
    if (st != MG_OK) return st;
    const int64_t n = std::min<int64_t>(std::min<int64_t>(steps, cap), kDtHistory);
    const double *hist = reinterpret_cast<const double *>(reinterpret_cast<const char *>(ctx->d_sp) + offsetof(StepParams, hist));
    // the last n steps in order: steps - n .. steps - 1, in at most two runs of the ring
    const int64_t first = steps - n;
    int64_t done = 0;
    while (done < n) {
        const int64_t at = (first + done) % kDtHistory;
        const int64_t run = std::min<int64_t>(n - done, kDtHistory - at);
        MG_CK(cudaMemcpyAsync(out + done, hist + at, run * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
        done += run;
    }
    MG_CK(cudaStreamSynchronize(ctx->stream));
    *n_out = n;
    return MG_OK;
}

mg_status mg_prepare(mg_context *ctx) {
    if (!ctx) return MG_ERR_ARG;
    mg_status st = require_ready(ctx);
    if (st != MG_OK) return st;
    // exchangeAtomFirst, clearForce, computeEam (src/simulation.cpp:137-145); the lattice passes assign
    // instead of accumulate, which is what clearForce + accumulate gives
    seq_compute_eam(ctx, false, false, 0, nullptr);
    if ((st = check_launch(ctx)) != MG_OK) return st;
    uint32_t bits = 0;
    if ((st = read_device_errors(ctx, &bits)) != MG_OK) return st;
    ctx->prepared = true;
    return status_from_bits(ctx, bits);
}

mg_status mg_simulate(mg_context *ctx, int64_t nsteps, int32_t sync) {
    if (!ctx || nsteps < 0) return MG_ERR_ARG;
    if (!ctx->prepared) { ctx->err = "mg_prepare must run before mg_simulate"; return MG_ERR_STATE; }
    mg_status st;
    if (ctx->vmax_stale) {
        launch_vmax_full(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->d_sp);
        ctx->vmax_stale = false;
    }
    if (ctx->timing) {
        const size_t need = static_cast<size_t>(nsteps) * (kNumTimers + 1);
        while (ctx->ev.size() < need) {
            cudaEvent_t e;
            MG_CK(cudaEventCreate(&e));
            ctx->ev.push_back(e);
        }
        // the same fusion pattern as the graphs: blocks of fuse_steps bodies, then single bodies
        const bool fuse = fusable(ctx) && nsteps >= 2;
        const int64_t k = fuse ? ctx->fuse_steps : 1, blocks = fuse ? nsteps / k : 0;
        for (int64_t i = 0; i < nsteps; i++) {
            Timer t{ctx, i};
            const bool in_block = i < blocks * k;
            const int64_t pos = i % k;
            if (in_block) set_body_buffers(ctx, k, pos);
            ctx->alt_bodies = in_block;
            seq_step(ctx, &t, in_block && pos > 0, in_block && pos < k - 1);
        }
        ctx->alt_bodies = false;
        set_body_buffers(ctx, 1, 0);
        if ((st = check_launch(ctx)) != MG_OK) return st;
        MG_CK(cudaStreamSynchronize(ctx->stream));
        ctx->timer_ms.assign(kNumTimers, 0.0);
        for (int64_t i = 0; i < nsteps; i++) {
            for (int k = 0; k < kNumTimers - 1; k++) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, ctx->ev[i * (kNumTimers + 1) + k], ctx->ev[i * (kNumTimers + 1) + k + 1]);
                ctx->timer_ms[k] += ms;
            }
        }
        ctx->timed_steps = nsteps;
    } else {
        if ((st = build_graph(ctx)) != MG_OK) return st;
        int64_t i = 0;
        if (fusable(ctx) && nsteps >= ctx->fuse_steps) {
            if ((st = build_graph_multi(ctx)) != MG_OK) return st;
            for (; i + ctx->fuse_steps <= nsteps; i += ctx->fuse_steps) MG_CK(cudaGraphLaunch(ctx->graph_multi, ctx->stream));
        }
        for (; i < nsteps; i++) MG_CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
    }
    ctx->energy_valid = false;
    if (sync) {
        uint32_t bits = 0;
        if ((st = read_device_errors(ctx, &bits)) != MG_OK) return st;
        return status_from_bits(ctx, bits);
    }
    return MG_OK;
}

mg_status mg_phase(mg_context *ctx, int32_t phase) {
    if (!ctx || phase < 0 || phase > 6) return MG_ERR_ARG;
    mg_status st = require_ready(ctx);
    if (st != MG_OK) return st;
    const LaunchCtx lc = ctx->lc();
    switch (phase) {
        case 0: seq_firststep(ctx, false, nullptr); break;
        case 1:
            launch_decide_scan(lc, ctx->g, ctx->s, ctx->in);
            launch_displaced_collect(lc, ctx->g, ctx->in);
            launch_far_clear(lc, ctx->g, ctx->in);
            launch_inter_manage(lc, ctx->g, ctx->s, ctx->in, MANAGE_DECIDE | MANAGE_CLEAR_GHOST, ctx->mixed());
            launch_far_mark(lc, ctx->g, ctx->in);
            break;
        case 2: launch_inter_manage(lc, ctx->g, ctx->s, ctx->in, MANAGE_EXCHANGE, ctx->mixed()); break;
        case 3: launch_inter_manage(lc, ctx->g, ctx->s, ctx->in, MANAGE_BORDER, ctx->mixed()); break;
        case 4: launch_ghost_copy(lc, ctx->g, ctx->s, ctx->mixed()); break;
        case 5: seq_compute_eam(ctx, false, false, 0, nullptr); break;
        case 6: launch_secondstep(lc, ctx->g, ctx->s, ctx->in, ctx->d_sp, true); break;
    }
    if ((st = check_launch(ctx)) != MG_OK) return st;
    uint32_t bits = 0;
    if ((st = read_device_errors(ctx, &bits)) != MG_OK) return st;
    ctx->energy_valid = false;
    ctx->vmax_stale = true;
    return status_from_bits(ctx, bits);
}

// simulation::collisionStep (src/simulation.cpp:208-217) enqueued on the context's stream
static mg_status enqueue_collision(mg_context *ctx, const int32_t lat[4], const double dir[3], double energy) {
    // atom::setv bounds (src/atom.cpp:477-482), one rank: the sub-box starts at 0
    const Geom &g = ctx->g;
    if (lat[3] < 0 || lat[3] > 1) { ctx->err = "PKA basis index must be 0 or 1"; return MG_ERR_ARG; }
    if ((lat[0] * 2) >= 0 && (lat[0] * 2) < g.bx && lat[1] >= 0 && lat[1] < g.by && lat[2] >= 0 && lat[2] < g.bz) {
        const int64_t kk = ((int64_t) (lat[2] + g.gz) * g.Sy + (lat[1] + g.gy)) * g.Sx + (lat[0] * 2 + g.gx) + lat[3];
        if (kk < 0 || kk >= g.n_slots) { ctx->err = "PKA slot outside the grid"; return MG_ERR_ARG; }
        launch_setv(ctx->lc(), g, ctx->s, kk, dir, energy);
        ctx->vmax_stale = true;
    }
    // exchangeInter, borderInter (the ghost list is not cleared here, as in the reference),
    // exchangeAtom, clearForce, computeEam
    launch_inter_manage(ctx->lc(), g, ctx->s, ctx->in, MANAGE_EXCHANGE | MANAGE_BORDER, ctx->mixed());
    seq_compute_eam(ctx, false, false, 0, nullptr);
    return check_launch(ctx);
}

mg_status mg_collision_step(mg_context *ctx, const int32_t lat[4], const double dir[3], double energy) {
    if (!ctx || !lat || !dir) return MG_ERR_ARG;
    mg_status st = require_ready(ctx);
    if (st != MG_OK) return st;
    if ((st = enqueue_collision(ctx, lat, dir, energy)) != MG_OK) return st;
    uint32_t bits = 0;
    if ((st = read_device_errors(ctx, &bits)) != MG_OK) return st;
    ctx->energy_valid = false;
    return status_from_bits(ctx, bits);
}

mg_status mg_rescale(mg_context *ctx, double t_set, uint64_t n_atoms) {
    if (!ctx || n_atoms < 2) return MG_ERR_ARG;
    launch_thermo(ctx->lc(), ctx->g, ctx->s, ctx->in, false, ctx->d_partials, ctx->n_partials, ctx->d_thermo);
    launch_rescale(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->d_thermo, t_set, n_atoms);
    ctx->vmax_stale = true;
    mg_status st = check_launch(ctx);
    if (st != MG_OK) return st;
    MG_CK(cudaStreamSynchronize(ctx->stream));
    return MG_OK;
}

// MDSimulation::beforeStep / postStep (frontend/md_simulation.cpp:40-111) around the loop body, all on
// the context's stream: stage changes set dt on the device, rescales and PKAs are kernels, steps are
// graph replays, thermo samples go to a device buffer read once at the end.
// OutputCopy::beforeCollision (frontend/io/output_copy.cpp:41-49): the state before the PKA as a
// one-frame file
static mg_status dump_origin(mg_context *ctx, uint64_t time_step) {
    mg_dump *d = nullptr;
    mg_status st = mg_dump_open(ctx, ctx->origin_path.c_str(), 0, 0, &d);
    if (st != MG_OK) return st;
    st = mg_dump_frame(d, time_step);
    std::string why = st != MG_OK ? mg_dump_last_error(d) : "";
    const mg_status st2 = mg_dump_close(d, nullptr);
    if (st == MG_OK) st = st2;
    if (st != MG_OK) ctx->err = "origin dump: " + (why.empty() ? ctx->err : why);
    return st;
}

mg_status mg_set_stage_output(mg_context *ctx, mg_dump *frames, uint64_t interval, const char *origin_path) {
    if (!ctx) return MG_ERR_ARG;
    ctx->stage_dump = frames;
    ctx->stage_dump_interval = frames ? interval : 0;
    ctx->origin_path = origin_path ? origin_path : "";
    return MG_OK;
}

extern "C++" {
namespace mg {
DumpSource dump_source(const mg_context *ctx) {
    return DumpSource{ctx->stream, static_cast<int64_t>(ctx->g.n_local) + ctx->in.cap, dump_scratch_ints(ctx->g)};
}
mg_status dump_pack(mg_context *ctx, mg_dump_record *out, unsigned long long *count, int *scratch, uint64_t step) {
    launch_dump_pack(ctx->lc(), ctx->g, ctx->s, ctx->in, out, count, scratch, step);
    return check_launch(ctx);
}
void dump_note_error(mg_context *ctx, const std::string &why) { ctx->err = why; }
void dump_detach(mg_context *ctx, const mg_dump *d) {
    if (ctx->stage_dump == d) {
        ctx->stage_dump = nullptr;
        ctx->stage_dump_interval = 0;
    }
}
}  // namespace mg
}  // extern "C++"

mg_status mg_run_stages(mg_context *ctx, const mg_stage *stages, int32_t n_stages, int64_t steps, double default_dt,
                        int64_t n_atoms, int32_t thermo_interval, mg_thermo_sample *samples, int64_t cap,
                        int64_t *n_samples) {
    if (!ctx || n_stages < 0 || (n_stages > 0 && !stages) || steps < 0 || n_atoms < 2 || thermo_interval < 0 ||
        cap < 0 || (cap > 0 && !samples) || !(default_dt > 0))
        return MG_ERR_ARG;
    if (!ctx->prepared) { ctx->err = "mg_prepare must run before mg_run_stages"; return MG_ERR_STATE; }
    for (int32_t k = 0; k < n_stages; k++) {
        const mg_stage &st = stages[k];
        if (st.steps < 0 || st.step_length < 0 || (st.rescales_set && (st.rescale_every < 1 || !(st.rescale_t > 0))) ||
            (st.collision_set && (st.collision_lat[3] < 0 || st.collision_lat[3] > 1))) {
            ctx->err = "stage " + std::to_string(k) + ": bad parameters";
            return MG_ERR_ARG;
        }
    }
    const int64_t want = thermo_interval ? steps / thermo_interval : 0;
    if (want > cap) { ctx->err = "sample buffer smaller than steps / thermo_interval"; return MG_ERR_ARG; }
    constexpr int kWords = 8;  // thermo words 0..5, steps, time
    if (want > ctx->n_samples_cap) {
        MG_CK(dalloc(ctx, &ctx->d_samples, static_cast<size_t>(want) * kWords));
        ctx->n_samples_cap = want;
    }
    mg_status st;
    if ((st = build_graph(ctx)) != MG_OK) return st;
    const LaunchCtx lc = ctx->lc();
    int64_t cur_stage_steps = 0, stage_len = 0, taken = 0;
    int32_t next = 0;
    const mg_stage *cur = nullptr;
    for (int64_t step = 0; step < steps; step++) {
        if (cur_stage_steps >= stage_len) {  // one stage change per step at most, as the reference does
            if (next >= n_stages) {
                ctx->err = "no more stages at step " + std::to_string(step);
                cudaStreamSynchronize(ctx->stream);
                return MG_ERR_STATE;
            }
            cur = &stages[next++];
            stage_len = cur->steps;
            cur_stage_steps = 0;
            set_dt(ctx, cur->step_length == 0.0 ? default_dt : cur->step_length);
        }
        if (cur->collision_set && cur_stage_steps + 1 == cur->collision_step) {
            if (!ctx->origin_path.empty() && (st = dump_origin(ctx, static_cast<uint64_t>(step))) != MG_OK) return st;
            if ((st = enqueue_collision(ctx, cur->collision_lat, cur->direction, cur->pka_energy)) != MG_OK) return st;
        }
        if (cur->rescales_set && cur_stage_steps % cur->rescale_every == 0) {
            launch_thermo(lc, ctx->g, ctx->s, ctx->in, false, ctx->d_partials, ctx->n_partials, ctx->d_thermo);
            launch_rescale(lc, ctx->g, ctx->s, ctx->in, ctx->d_thermo, cur->rescale_t, static_cast<uint64_t>(n_atoms));
            ctx->vmax_stale = true;
        }
        if (ctx->vmax_stale) {
            launch_vmax_full(lc, ctx->g, ctx->s, ctx->in, ctx->d_sp);
            ctx->vmax_stale = false;
        }
        // a fused graph of fuse_steps bodies when none of them has an event inside the run: no stage
        // change, PKA or rescale before bodies 1 .. k-1, no dump or thermo sample after bodies 0 .. k-2
        const int64_t k = ctx->fuse_steps;
        bool fused = fusable(ctx) && step + k <= steps;
        for (int64_t j = 1; fused && j < k; j++) {
            const int64_t css = cur_stage_steps + j, sj = step + j;
            if (css >= stage_len || (cur->collision_set && css + 1 == cur->collision_step) ||
                (cur->rescales_set && css % cur->rescale_every == 0))
                fused = false;
            const int64_t before = sj;  // body j - 1 ends at step number sj (1-based)
            if ((ctx->stage_dump && ctx->stage_dump_interval && before % ctx->stage_dump_interval == 0) ||
                (thermo_interval && before % thermo_interval == 0))
                fused = false;
        }
        if (fused) {
            if ((st = build_graph_multi(ctx)) != MG_OK) return st;
            MG_CK(cudaGraphLaunch(ctx->graph_multi, ctx->stream));
            cur_stage_steps += k - 1;
            step += k - 1;
        } else {
            MG_CK(cudaGraphLaunch(ctx->graph_exec, ctx->stream));
        }
        cur_stage_steps++;
        if (ctx->stage_dump && ctx->stage_dump_interval && (step + 1) % ctx->stage_dump_interval == 0) {
            if ((st = mg_dump_frame(ctx->stage_dump, static_cast<uint64_t>(step + 1))) != MG_OK) {
                ctx->err = std::string("dump: ") + mg_dump_last_error(ctx->stage_dump);
                return st;
            }
        }
        if (thermo_interval && (step + 1) % thermo_interval == 0) {
            double *rec = ctx->d_samples + kWords * taken;
            launch_thermo(lc, ctx->g, ctx->s, ctx->in, false, ctx->d_partials, ctx->n_partials, rec);
            launch_clock_sample(lc, ctx->d_sp, rec + 6);
            taken++;
        }
    }
    if ((st = check_launch(ctx)) != MG_OK) return st;
    std::vector<double> h(static_cast<size_t>(taken) * kWords);
    if (taken) MG_CK(cudaMemcpyAsync(h.data(), ctx->d_samples, h.size() * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    const double to_t = kMvv2e / (static_cast<double>(3 * n_atoms - 3) * kBoltz);
    for (int64_t k = 0; k < taken; k++) {
        const double *r = &h[kWords * k];
        samples[k].step = static_cast<int64_t>(r[6]);
        samples[k].time_ps = r[7];
        samples[k].mvv = r[0];
        samples[k].temperature = r[0] * to_t;
    }
    if (n_samples) *n_samples = taken;
    ctx->energy_valid = false;
    uint32_t bits = 0;
    if ((st = read_device_errors(ctx, &bits)) != MG_OK) return st;
    return status_from_bits(ctx, bits);
}

mg_status mg_thermo(mg_context *ctx, int32_t with_energy, mg_thermo_out *out) {
    if (!ctx || !out) return MG_ERR_ARG;
    mg_status st;
    if (with_energy) {
        if ((st = require_ready(ctx)) != MG_OK) return st;
        launch_energy(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->pt, ctx->mixed());
        launch_inter_energy(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->pt, ctx->mixed());
        ctx->energy_valid = true;
    }
    launch_thermo(ctx->lc(), ctx->g, ctx->s, ctx->in, with_energy != 0, ctx->d_partials, ctx->n_partials, ctx->d_thermo);
    if ((st = check_launch(ctx)) != MG_OK) return st;
    double h[6];
    int cnt[CNT_WORDS];
    MG_CK(cudaMemcpyAsync(h, ctx->d_thermo, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaMemcpyAsync(cnt, ctx->in.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    std::memset(out, 0, sizeof(*out));
    out->mvv = h[0];
    out->kinetic_energy = h[0] / 2;
    out->force_sum[0] = h[1]; out->force_sum[1] = h[2]; out->force_sum[2] = h[3];
    out->potential_energy = with_energy ? h[4] : 0.0;
    out->n_vacancy = static_cast<int64_t>(h[5]);
    out->n_inter = cnt[CNT_INTER];
    out->n_ghost_inter = cnt[CNT_GHOST];
    out->device_errors = static_cast<uint32_t>(cnt[CNT_ERRORS]);
    return MG_OK;
}

mg_status mg_download_energies(mg_context *ctx, double *per_slot, int64_t n_slots, double *per_inter,
                               int64_t inter_cap) {
    if (!ctx || !per_slot || n_slots != ctx->g.n_slots) return MG_ERR_ARG;
    if (!ctx->energy_valid) { ctx->err = "no energy pass since the last state change"; return MG_ERR_STATE; }
    MG_CK(cudaMemcpyAsync(per_slot, ctx->s.e, n_slots * sizeof(double), cudaMemcpyDeviceToHost, ctx->stream));
    int cnt[CNT_WORDS];
    MG_CK(cudaMemcpyAsync(cnt, ctx->in.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    // local slots only: ghosts and vacancies are reported as 0
    std::vector<int8_t> ty(n_slots);
    MG_CK(cudaMemcpy(ty.data(), ctx->s.type, n_slots, cudaMemcpyDeviceToHost));
    const Geom &g = ctx->g;
    for (int64_t s = 0; s < n_slots; s++) {
        const int64_t X = s % g.Sx, r = s / g.Sx, Y = r % g.Sy, Z = r / g.Sy;
        const bool local = X >= g.gx && X < g.gx + g.bx && Y >= g.gy && Y < g.gy + g.by && Z >= g.gz && Z < g.gz + g.bz;
        if (!local || ty[s] < 0) per_slot[s] = 0.0;
    }
    const int64_t m = std::min<int64_t>(cnt[CNT_INTER], per_inter ? inter_cap : 0);
    if (m > 0) MG_CK(cudaMemcpy(per_inter, ctx->in.e, m * sizeof(double), cudaMemcpyDeviceToHost));
    return MG_OK;
}

mg_status mg_clear_errors(mg_context *ctx) {
    if (!ctx) return MG_ERR_ARG;
    int z = 0;
    MG_CK(cudaMemcpyAsync(ctx->in.cnt + CNT_ERRORS, &z, sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    return MG_OK;
}

// One loop body from and to the host slot array with the copies out overlapped by the copies in (fixed
// dt, no inter atoms in; the host link carries both directions at once). The in-chunks arrive bottom to
// top into a kept input buffer. Each is unpacked and takes its firststep, decide's own-site case
// (launch_spec_decide) and its in-plane ghost copy. A density slab runs once every plane within 3 of it
// has arrived, a force slab once the density slabs beside it have run, and its finished planes are packed
// and copied out at once while later chunks are still coming in. The thin slabs at the periodic z seam
// (two of 4 planes at each end) wait for the ghost planes, copied after the last chunk. Per atom the
// kernels and their order are those of the unpipelined path, so the result is bit-identical to it. If a
// chunk's decide met a displaced atom that does not go straight back to its own site, the step is void:
// it runs again in full from the kept input, as mg_upload + one loop body + mg_download would.
// S >= 6 in-chunks and 6 <= SS <= bz / 4 density slabs, at least 32 sites of a parity per plane.
static mg_status step_host_overlapped(mg_context *ctx, mg_atom_element *atoms, mg_atom_element *inter,
                                      int64_t inter_cap, int64_t *n_inter, int S, int SS) {
    const Geom &g = ctx->g;
    if (!ctx->copy_in) MG_CK(cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
    if (!ctx->copy_out) MG_CK(cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
    const size_t n_ev = static_cast<size_t>(S + SS + 8);
    while (ctx->pipe_ev.size() < n_ev) {
        cudaEvent_t e;
        MG_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->pipe_ev.push_back(e);
    }
    mg_status st;
    if ((st = ensure_aos(ctx)) != MG_OK) return st;
    if (!ctx->d_aos_in) MG_CK(dalloc(ctx, &ctx->d_aos_in, static_cast<size_t>(g.n_slots)));
    const LaunchCtx lc = ctx->lc();
    const bool mx = ctx->mixed();
    const int K = g.bz;
    const int64_t plane = static_cast<int64_t>(g.Sx) * g.Sy;  // slots per z plane
    const int pp = g.by * g.nxh;                               // sites of one parity per local plane
    const size_t rec = sizeof(mg_atom_element);
    size_t ev = 0;
    // in-chunks of whole planes: three thin ones (4 planes) first, so that the first slabs start early,
    // then even ones, and a thin last one
    auto local_plane_bound = [&](int c) {
        if (c == S) return K;
        if (c == S - 1) return K - 4;
        if (c <= 3) return 4 * c;
        return 12 + static_cast<int>((static_cast<int64_t>(c - 3) * (K - 16)) / (S - 4));
    };
    // density and force slabs: kb[c] local planes, u[c] sites (whole 32-site groups). Three thin ones at
    // the bottom and two at the top (4 planes), even ones of at least 4 planes between
    std::vector<int> kb(SS + 1), u(SS + 1);
    for (int c = 0; c <= SS; c++) {
        if (c <= 3) kb[c] = 4 * c;
        else if (c >= SS - 2) kb[c] = K - 4 * (SS - c);
        else kb[c] = 12 + static_cast<int>((static_cast<int64_t>(c - 3) * (K - 20)) / (SS - 5));
        u[c] = c == SS ? g.n_local_half : static_cast<int>(((static_cast<int64_t>(kb[c]) * pp) >> 5) << 5);
    }
    auto last_plane = [&](int c) { return (u[c + 1] - 1) / pp; };    // the plane of slab c's last site
    auto planes_below = [&](int c) { return u[c] / pp; };           // planes wholly below u[c]
    auto planes_from = [&](int c) { return (u[c] + pp - 1) / pp; };  // first plane wholly at or above u[c]

    // head: the copies wait for everything already on the library stream
    MG_CK(cudaEventRecord(ctx->pipe_ev[ev], ctx->stream));
    MG_CK(cudaStreamWaitEvent(ctx->copy_in, ctx->pipe_ev[ev++], 0));
    launch_set_counts(lc, ctx->in, 0);
    launch_step_head(lc, ctx->d_sp);
    launch_far_clear(lc, g, ctx->in);  // the previous far list's marks, which decide clears
    launch_spec_begin(lc, ctx->in);
    std::vector<size_t> in_ev(S);
    std::vector<int64_t> cs0(S), cs1(S);
    for (int c = 0; c < S; c++) {
        const int z0 = c == 0 ? 0 : g.gz + local_plane_bound(c);
        const int z1 = c == S - 1 ? g.Sz : g.gz + local_plane_bound(c + 1);
        cs0[c] = z0 * plane;
        cs1[c] = z1 * plane;
        MG_CK(cudaMemcpyAsync(ctx->d_aos_in + cs0[c], atoms + cs0[c], static_cast<size_t>(cs1[c] - cs0[c]) * rec,
                              cudaMemcpyHostToDevice, ctx->copy_in));
        in_ev[c] = ev;
        MG_CK(cudaEventRecord(ctx->pipe_ev[ev++], ctx->copy_in));
    }
    // out: pack the slot planes [z0, z1) and copy them on copy_out
    auto flush = [&](int z0, int z1) -> mg_status {
        if (z1 <= z0) return MG_OK;
        const int64_t s0 = z0 * plane, s1 = z1 * plane;
        launch_pack_aos(lc, g, ctx->d_aos, ctx->s, PACK_ALL, mx, static_cast<int>(s0), static_cast<int>(s1));
        MG_CK(cudaEventRecord(ctx->pipe_ev[ev], ctx->stream));
        MG_CK(cudaStreamWaitEvent(ctx->copy_out, ctx->pipe_ev[ev++], 0));
        MG_CK(cudaMemcpyAsync(atoms + s0, ctx->d_aos + s0, static_cast<size_t>(s1 - s0) * rec, cudaMemcpyDeviceToHost,
                              ctx->copy_out));
        return MG_OK;
    };
    auto rho_slab = [&](int c) { launch_lat_rho_sites(lc, g, ctx->s, ctx->in, ctx->pt, mx, u[c], u[c + 1], true); };
    auto force_slab = [&](int c) {
        launch_lat_force_sites(lc, g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, true, mx, u[c], u[c + 1], true);
    };
    int next_rho = 1, next_force = 2;
    int df_hi = planes_from(1);                 // in-plane ghosts of planes [planes_from(1), df_hi) have their df
    const int out_lo = g.gz + planes_from(2);   // slot planes [out_lo, out_hi) are on their way out
    int out_hi = out_lo;
    for (int c = 0; c < S; c++) {
        MG_CK(cudaStreamWaitEvent(ctx->stream, ctx->pipe_ev[in_ev[c]], 0));
        launch_unpack_aos(lc, g, ctx->d_aos_in, ctx->s, ctx->in, ctx->types_ok_mask, mx, static_cast<int>(cs0[c]),
                          static_cast<int>(cs1[c]));
        const int k0 = c == 0 ? 0 : local_plane_bound(c), k1 = local_plane_bound(c + 1);
        const int t0 = k0 * g.by * g.bx, t1 = k1 * g.by * g.bx;
        launch_firststep(lc, g, ctx->s, ctx->in, ctx->d_sp, true, t0, t1);
        launch_spec_decide(lc, g, ctx->s, ctx->in, t0, t1);
        launch_ghost_copy_planes(lc, g, ctx->s, k0, k1);
        // slabs 1 .. SS - 2 in order once the planes within 3 of them are in; then the forces of slabs
        // 2 .. SS - 3 whose neighbour slabs have their density, and their finished planes go out
        while (next_rho <= SS - 2 && last_plane(next_rho) + 3 < k1) {
            rho_slab(next_rho);
            const int hi = planes_below(next_rho + 1);
            launch_ghost_df_planes(lc, g, ctx->s, ctx->in, mx, df_hi, hi);
            df_hi = std::max(df_hi, hi);
            next_rho++;
            while (next_force <= SS - 3 && next_force + 1 < next_rho) {
                force_slab(next_force);
                const int z_to = g.gz + planes_below(next_force + 1);
                if ((st = flush(out_hi, z_to)) != MG_OK) return st;
                out_hi = std::max(out_hi, z_to);
                next_force++;
            }
        }
    }
    if (next_rho != SS - 1 || next_force != SS - 2) {
        ctx->err = "overlapped host step: slab schedule incomplete";
        return MG_ERR_STATE;
    }
    // the seam: ghost planes, the end slabs' density and ghost df, then their forces
    launch_ghost_copy_planes(lc, g, ctx->s, -1, -1);
    rho_slab(0);
    rho_slab(SS - 1);
    launch_ghost_df_planes(lc, g, ctx->s, ctx->in, mx, 0, planes_from(1));
    launch_ghost_df_planes(lc, g, ctx->s, ctx->in, mx, df_hi, K);
    launch_ghost_df_planes(lc, g, ctx->s, ctx->in, mx, -1, -1);
    if (mx) launch_skin_advance(lc, ctx->s);  // after the last density slab
    force_slab(1);
    force_slab(0);
    if ((st = flush(0, out_lo)) != MG_OK) return st;
    force_slab(SS - 2);
    force_slab(SS - 1);
    if ((st = flush(out_hi, g.Sz)) != MG_OK) return st;
    seq_eam_force_tail(ctx, true, nullptr);
    if ((st = check_launch(ctx)) != MG_OK) return st;

    int cnt[CNT_WORDS];
    MG_CK(cudaMemcpyAsync(cnt, ctx->in.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->copy_out));
    ctx->prepared = true;
    ctx->vmax_stale = true;
    ctx->energy_valid = false;
    if (cnt[CNT_SPEC_VOID]) {
        // the whole loop body again from the kept input (the step head has run once already)
        launch_unpack_aos(lc, g, ctx->d_aos_in, ctx->s, ctx->in, ctx->types_ok_mask, mx);
        launch_set_counts(lc, ctx->in, 0);
        seq_firststep(ctx, true, nullptr);
        seq_compute_eam(ctx, true, true, MANAGE_DECIDE | MANAGE_CLEAR_GHOST | MANAGE_EXCHANGE | MANAGE_BORDER, nullptr);
        if ((st = check_launch(ctx)) != MG_OK) return st;
        if ((st = mg_download(ctx, atoms, g.n_slots, inter, inter_cap, n_inter)) != MG_OK) return st;
        uint32_t bits = 0;
        if ((st = read_device_errors(ctx, &bits)) != MG_OK) return st;
        return status_from_bits(ctx, bits);
    }
    *n_inter = 0;
    return status_from_bits(ctx, static_cast<uint32_t>(cnt[CNT_ERRORS]));
}

// One loop body from and to the host slot array with the copies overlapped by the step (fixed dt, no
// inter atoms in), for boxes too thin for the overlapped path above. The slot grid is cut into z-slabs
// of whole planes:
//   in:  slab c is copied in on copy_in while slab c - 1 is unpacked and takes its firststep;
//   out: density and force run slab by slab; once a slab's planes are final they are packed and copied
//        out on copy_out while the next slabs compute.
// Per atom the kernels are those of mg_upload + mg_simulate + mg_download, so the result is
// bit-identical. The host reads the inter-atom count after decide: if decide moved atoms off the
// lattice, their density and force passes follow the lattice passes, so the step finishes unsplit
// and the state goes out in one download.
static mg_status step_host_pipelined(mg_context *ctx, mg_atom_element *atoms, mg_atom_element *inter, int64_t inter_cap,
                                     int64_t *n_inter) {
    const Geom &g = ctx->g;
    const int S = std::min(ctx->host_chunks, g.bz);
    {
        // density slabs about twice as many as the chunks: thinner slabs keep the copies out close
        // behind the copies in
        const int SS = std::min(2 * S, g.bz / 4);
        if (S >= 6 && SS >= 6 && g.by * g.nxh >= 32) return step_host_overlapped(ctx, atoms, inter, inter_cap, n_inter, S, SS);
    }
    if (!ctx->copy_in) MG_CK(cudaStreamCreateWithFlags(&ctx->copy_in, cudaStreamNonBlocking));
    if (!ctx->copy_out) MG_CK(cudaStreamCreateWithFlags(&ctx->copy_out, cudaStreamNonBlocking));
    const size_t n_ev = static_cast<size_t>(2 * S + 4);
    while (ctx->pipe_ev.size() < n_ev) {
        cudaEvent_t e;
        MG_CK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        ctx->pipe_ev.push_back(e);
    }
    mg_status st;
    if ((st = ensure_aos(ctx)) != MG_OK) return st;
    const LaunchCtx lc = ctx->lc();
    const bool mx = ctx->mixed();
    const int64_t plane = static_cast<int64_t>(g.Sx) * g.Sy;  // slots per z plane
    const size_t rec = sizeof(mg_atom_element);
    size_t ev = 0;
    // copy-in chunks: uniform, but the last one thin (4 planes), since its unpack and firststep are not
    // hidden behind a copy
    auto local_plane_bound = [&](int c) {
        if (S >= 3 && g.bz >= 8 * S) {
            if (c == S) return g.bz;
            if (c == S - 1) return g.bz - 4;
            return static_cast<int>((static_cast<int64_t>(c) * (g.bz - 4)) / (S - 1));
        }
        return static_cast<int>((static_cast<int64_t>(c) * g.bz) / S);
    };

    // in: the copies wait for everything already on the library stream
    MG_CK(cudaEventRecord(ctx->pipe_ev[ev], ctx->stream));
    MG_CK(cudaStreamWaitEvent(ctx->copy_in, ctx->pipe_ev[ev++], 0));
    launch_set_counts(lc, ctx->in, 0);
    launch_step_head(lc, ctx->d_sp);
    for (int c = 0; c < S; c++) {
        const int z0 = c == 0 ? 0 : g.gz + local_plane_bound(c);
        const int z1 = c == S - 1 ? g.Sz : g.gz + local_plane_bound(c + 1);
        const int64_t s0 = z0 * plane, s1 = z1 * plane;
        MG_CK(cudaMemcpyAsync(ctx->d_aos + s0, atoms + s0, static_cast<size_t>(s1 - s0) * rec, cudaMemcpyHostToDevice,
                              ctx->copy_in));
        MG_CK(cudaEventRecord(ctx->pipe_ev[ev], ctx->copy_in));
        MG_CK(cudaStreamWaitEvent(ctx->stream, ctx->pipe_ev[ev++], 0));
        launch_unpack_aos(lc, g, ctx->d_aos, ctx->s, ctx->in, ctx->types_ok_mask, mx, static_cast<int>(s0),
                          static_cast<int>(s1));
        const int k0 = std::max(z0 - g.gz, 0), k1 = std::min(z1 - g.gz, g.bz);
        if (k1 > k0) launch_firststep(lc, g, ctx->s, ctx->in, ctx->d_sp, true, k0 * g.by * g.bx, k1 * g.by * g.bx);
    }
    launch_inter_firststep(lc, ctx->in, ctx->d_sp);
    seq_eam_lists(ctx, true, MANAGE_DECIDE | MANAGE_CLEAR_GHOST | MANAGE_EXCHANGE | MANAGE_BORDER, nullptr);
    // whether decide left inter atoms: they add density and force after the lattice passes, which
    // orders the whole density pass before any force (and the slabs' early copies would be stale)
    int n_inter_now = 0;
    MG_CK(cudaMemcpyAsync(&n_inter_now, ctx->in.cnt + CNT_INTER, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    if ((st = check_launch(ctx)) != MG_OK) return st;
    if (n_inter_now > 0) {  // the unpipelined remainder, then one download of everything
        seq_eam_rho(ctx, nullptr);
        launch_lat_force(lc, g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, true, mx, false, false, true);
        seq_eam_force_tail(ctx, true, nullptr);
        if ((st = check_launch(ctx)) != MG_OK) return st;
        ctx->prepared = true;
        ctx->vmax_stale = true;
        ctx->energy_valid = false;
        if ((st = mg_download(ctx, atoms, g.n_slots, inter, inter_cap, n_inter)) != MG_OK) return st;
        uint32_t bits = 0;
        if ((st = read_device_errors(ctx, &bits)) != MG_OK) return st;
        return status_from_bits(ctx, bits);
    }

    // out: pack the planes [z0, z1) once final and copy them on copy_out
    auto flush = [&](int z0, int z1) -> mg_status {
        if (z1 <= z0) return MG_OK;
        const int64_t s0 = z0 * plane, s1 = z1 * plane;
        launch_pack_aos(lc, g, ctx->d_aos, ctx->s, PACK_ALL, mx, static_cast<int>(s0), static_cast<int>(s1));
        MG_CK(cudaEventRecord(ctx->pipe_ev[ev], ctx->stream));
        MG_CK(cudaStreamWaitEvent(ctx->copy_out, ctx->pipe_ev[ev++], 0));
        MG_CK(cudaMemcpyAsync(atoms + s0, ctx->d_aos + s0, static_cast<size_t>(s1 - s0) * rec, cudaMemcpyDeviceToHost,
                              ctx->copy_out));
        return MG_OK;
    };
    // Density and force in S z-slabs of sites. A site's neighbours lie within 3 planes, so with slabs of
    // at least 4 planes the force of slab c needs the density of slabs c - 1 .. c + 1 only, and the
    // ghost planes (periodic images of the top and bottom slabs) only for slabs 0 and S - 1. Order:
    // rho 0, rho 1, then per c = 1 .. S - 2 rho c + 1 and force c (its planes go out), then the ghost
    // planes' df, force S - 1 and force 0. Without inter atoms every site's df is final after its
    // density slab (dF/drho is fused), and the in-plane ghosts' df after that plane's density.
    const int64_t per_plane = static_cast<int64_t>(g.by) * g.nxh;  // sites of one parity per local plane
    const int SS = std::min(S, g.bz / 4);
    if (SS < 3) {
        seq_eam_rho(ctx, nullptr);
        if ((st = flush(0, g.gz)) != MG_OK) return st;
        launch_lat_force(lc, g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, true, mx, false, false, true);
        if ((st = flush(g.gz, g.Sz)) != MG_OK) return st;
    } else {
        // slabs 0 .. 2 thin (4 planes): the first copy out waits for their density and slab 1's force
        std::vector<int> kb(SS + 1);
        const int thin = (SS >= 6 && g.bz >= 8 * SS) ? 3 : 0;
        for (int c = 0; c <= SS; c++)
            kb[c] = c <= thin ? 4 * c
                              : 4 * thin + static_cast<int>((static_cast<int64_t>(c - thin) * (g.bz - 4 * thin)) / (SS - thin));
        std::vector<int> u(SS + 1);
        for (int c = 0; c <= SS; c++)
            u[c] = c == SS ? g.n_local_half : static_cast<int>(((kb[c] * per_plane) >> 5) << 5);
        auto full_planes = [&](int c) { return c == SS ? g.bz : static_cast<int>(u[c] / per_plane); };  // below u[c]
        int df_done = 0;  // local planes whose in-plane ghosts have their df
        auto rho_slab = [&](int c) {
            launch_lat_rho_sites(lc, g, ctx->s, ctx->in, ctx->pt, mx, u[c], u[c + 1], true);
            const int k = full_planes(c + 1);
            launch_ghost_df_planes(lc, g, ctx->s, ctx->in, mx, df_done, k);
            df_done = k;
        };
        rho_slab(0);
        rho_slab(1);
        // planes of slabs 1 .. S - 2 go out after their force; the plane cut by u[1] waits for slab 0
        int z_done = g.gz + (u[1] % per_plane ? full_planes(1) + 1 : full_planes(1));
        const int z_first = z_done;
        for (int c = 1; c <= SS - 2; c++) {
            rho_slab(c + 1);
            launch_lat_force_sites(lc, g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, true, mx, u[c], u[c + 1], true);
            const int z_to = g.gz + full_planes(c + 1);
            if ((st = flush(z_done, z_to)) != MG_OK) return st;
            z_done = std::max(z_done, z_to);
        }
        if (mx) launch_skin_advance(lc, ctx->s);  // after the last density slab (no firststep since)
        launch_ghost_df_planes(lc, g, ctx->s, ctx->in, mx, -1, -1);
        launch_lat_force_sites(lc, g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, true, mx, u[SS - 1], u[SS], true);
        if ((st = flush(z_done, g.Sz)) != MG_OK) return st;
        launch_lat_force_sites(lc, g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, true, mx, u[0], u[1], true);
        if ((st = flush(0, z_first)) != MG_OK) return st;
    }
    seq_eam_force_tail(ctx, true, nullptr);
    if ((st = check_launch(ctx)) != MG_OK) return st;

    int cnt[CNT_WORDS];
    MG_CK(cudaMemcpyAsync(cnt, ctx->in.cnt, sizeof(cnt), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->copy_out));
    ctx->prepared = true;
    ctx->vmax_stale = true;
    ctx->energy_valid = false;
    *n_inter = cnt[CNT_INTER];  // 0: checked after decide
    return status_from_bits(ctx, static_cast<uint32_t>(cnt[CNT_ERRORS]));
}

mg_status mg_set_step_fusion(mg_context *ctx, int32_t steps_per_graph) {
    if (!ctx || steps_per_graph < 0 || steps_per_graph > 256) return MG_ERR_ARG;
    ctx->fuse_steps = steps_per_graph;
    if (ctx->graph_multi) { cudaGraphExecDestroy(ctx->graph_multi); ctx->graph_multi = nullptr; }
    return MG_OK;
}

mg_status mg_set_neighbour_skin(mg_context *ctx, double skin) {
    if (!ctx || !(skin >= 0.0) || skin > ctx->g.a0) return MG_ERR_ARG;
    set_skin(ctx->g, skin);
    launch_skin_dirty(ctx->lc(), ctx->s);
    ctx->graph_stale = true;  // the captured kernels hold the old geometry
    ctx->gen++;
    if (ctx->graph_multi) { cudaGraphExecDestroy(ctx->graph_multi); ctx->graph_multi = nullptr; }
    return check_launch(ctx);
}

mg_status mg_skin_stats(mg_context *ctx, int64_t *passes, int64_t *rebuilds) {
    if (!ctx || !passes || !rebuilds) return MG_ERR_ARG;
    SkinState k;
    MG_CK(cudaMemcpyAsync(&k, ctx->s.skin, sizeof(k), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    *passes = static_cast<int64_t>(k.passes);
    *rebuilds = static_cast<int64_t>(k.rebuilds);
    return MG_OK;
}

mg_status mg_set_host_pipeline(mg_context *ctx, int32_t chunks) {
    if (!ctx || chunks < 0) return MG_ERR_ARG;
    ctx->host_chunks = chunks;
    return MG_OK;
}

mg_status mg_step_host(mg_context *ctx, mg_atom_element *atoms, int64_t n_slots, mg_atom_element *inter,
                       int64_t inter_cap, int64_t *n_inter, int64_t nsteps) {
    if (!ctx || !atoms || !n_inter) return MG_ERR_ARG;
    if (nsteps == 1 && *n_inter == 0 && n_slots == ctx->g.n_slots && ctx->host_chunks >= 2 && ctx->dx_max <= 0.0 &&
        !ctx->timing && ctx->pot_ready)
        return step_host_pipelined(ctx, atoms, inter, inter_cap, n_inter);
    mg_status st = mg_upload(ctx, atoms, n_slots, inter, std::min<int64_t>(*n_inter, inter_cap));
    if (st != MG_OK) return st;
    ctx->prepared = true;  // the host state carries forces from its previous computeEam
    if ((st = mg_simulate(ctx, nsteps, 0)) != MG_OK) return st;
    return mg_download(ctx, atoms, n_slots, inter, inter_cap, n_inter);
}

mg_status mg_ws_map(mg_context *ctx, const double *xyz, int64_t n, int64_t *coords, uint32_t *flags, int64_t *index) {
    if (!ctx || !xyz || !coords || !flags || !index || n < 0) return MG_ERR_ARG;
    if (n == 0) return MG_OK;
    if (n > ctx->ws_cap) {
        MG_CK(dalloc(ctx, &ctx->d_ws_xyz, 3 * (size_t) n));
        MG_CK(dalloc(ctx, &ctx->d_ws_coords, 3 * (size_t) n));
        MG_CK(dalloc(ctx, &ctx->d_ws_flags, (size_t) n));
        MG_CK(dalloc(ctx, &ctx->d_ws_index, (size_t) n));
        ctx->ws_cap = n;
    }
    MG_CK(cudaMemcpyAsync(ctx->d_ws_xyz, xyz, 3 * n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    launch_ws_map(ctx->lc(), ctx->g, ctx->d_ws_xyz, n, ctx->d_ws_coords, ctx->d_ws_flags, ctx->d_ws_index);
    mg_status st = check_launch(ctx);
    if (st != MG_OK) return st;
    MG_CK(cudaMemcpyAsync(coords, ctx->d_ws_coords, 3 * n * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaMemcpyAsync(flags, ctx->d_ws_flags, n * sizeof(uint32_t), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaMemcpyAsync(index, ctx->d_ws_index, n * sizeof(int64_t), cudaMemcpyDeviceToHost, ctx->stream));
    MG_CK(cudaStreamSynchronize(ctx->stream));
    return MG_OK;
}

// Autotuner: times each gather kernel of the current precision for every (thread order, block size)
// on the resident state and keeps the fastest; results are cached per (box, precision) for the process.
namespace {
struct TuneKey {
    int cells[3], precision;
    bool operator==(const TuneKey &o) const {
        return cells[0] == o.cells[0] && cells[1] == o.cells[1] && cells[2] == o.cells[2] && precision == o.precision;
    }
};
std::vector<std::pair<TuneKey, std::array<int, 6>>> g_tune_cache;
std::mutex g_tune_mutex;
}  // namespace

mg_status mg_autotune(mg_context *ctx, int32_t reps, int32_t out[6]) {
    if (!ctx) return MG_ERR_ARG;
    if (!ctx->prepared) { ctx->err = "mg_prepare must run before mg_autotune"; return MG_ERR_STATE; }
    const int p = ctx->precision;
    const TuneKey key{{ctx->g.cells[0], ctx->g.cells[1], ctx->g.cells[2]}, p};
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        for (auto &kv : g_tune_cache) {
            if (kv.first == key) {
                for (int k = 0; k < 2; k++)
                    for (int c = 0; c < 3; c++) ctx->tune[p][k][c] = kv.second[3 * k + c];
                if (out) for (int k = 0; k < 6; k++) out[k] = kv.second[k];
                ctx->graph_stale = true;
                ctx->gen++;
                return MG_OK;
            }
        }
    }
    if (reps < 1) reps = 3;
    cudaEvent_t e0, e1;
    MG_CK(cudaEventCreate(&e0));
    MG_CK(cudaEventCreate(&e1));
    const int blocks[3] = {128, 256, 512}, apts[3] = {1, 2, 4};
    std::array<int, 6> best{};
    for (int kern = 0; kern < 2; kern++) {
        float best_ms = 1e30f;
        for (int order = 0; order < 2; order++) {
            for (int b : blocks) for (int apt : apts) {
                ctx->tune[p][kern][0] = order;
                ctx->tune[p][kern][1] = b;
                ctx->tune[p][kern][2] = apt;
                const LaunchCtx lc = ctx->lc();
                auto run = [&]() {
                    if (kern == 0) launch_lat_rho(lc, ctx->g, ctx->s, ctx->in, ctx->pt, ctx->mixed(), false);
                    else launch_lat_force(lc, ctx->g, ctx->s, ctx->in, ctx->pt, ctx->d_sp, false, ctx->mixed(), false);
                };
                run();  // warm
                cudaEventRecord(e0, ctx->stream);
                for (int r = 0; r < reps; r++) run();
                cudaEventRecord(e1, ctx->stream);
                MG_CK(cudaEventSynchronize(e1));
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best_ms) { best_ms = ms; best[3 * kern] = order; best[3 * kern + 1] = b; best[3 * kern + 2] = apt; }
            }
        }
        for (int c = 0; c < 3; c++) ctx->tune[p][kern][c] = best[3 * kern + c];
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    mg_status st = check_launch(ctx);
    if (st != MG_OK) return st;
    {
        std::lock_guard<std::mutex> lock(g_tune_mutex);
        g_tune_cache.push_back({key, best});
    }
    if (out) for (int k = 0; k < 6; k++) out[k] = best[k];
    ctx->graph_stale = true;
    ctx->gen++;  // the captured graph holds the old launch shapes
    return MG_OK;
}

mg_status mg_set_tuning(mg_context *ctx, const int32_t tune[6]) {
    if (!ctx || !tune) return MG_ERR_ARG;
    for (int k = 0; k < 2; k++) {
        const int order = tune[3 * k], b = tune[3 * k + 1], apt = tune[3 * k + 2];
        if ((order != 0 && order != 1) || (b != 128 && b != 256 && b != 512) || apt < 1 || apt > 64) return MG_ERR_ARG;
    }
    for (int k = 0; k < 2; k++)
        for (int c = 0; c < 3; c++) ctx->tune[ctx->precision][k][c] = tune[3 * k + c];
    ctx->graph_stale = true;
    ctx->gen++;
    return MG_OK;
}

mg_status mg_enable_timing(mg_context *ctx, int32_t on) {
    if (!ctx) return MG_ERR_ARG;
    ctx->timing = on != 0;
    return MG_OK;
}

mg_status mg_kernel_times(const mg_context *ctx, double *ms, int32_t cap, int32_t *n, const char **names) {
    if (!ctx || !n) return MG_ERR_ARG;
    *n = kNumTimers - 1;
    for (int k = 0; k < kNumTimers - 1 && k < cap; k++) {
        if (ms) ms[k] = ctx->timed_steps ? ctx->timer_ms.size() > (size_t) k ? ctx->timer_ms[k] / ctx->timed_steps : 0.0 : 0.0;
        if (names) names[k] = kTimerNames[k];
    }
    return MG_OK;
}

mg_status mg_launches_per_step(const mg_context *ctx, int32_t *n) {
    if (!ctx || !n) return MG_ERR_ARG;
    *n = ctx->launches_per_step > 0 ? ctx->launches_per_step : kLaunchesPerStep;
    return MG_OK;
}

void *mg_stream(const mg_context *ctx) { return ctx ? (void *) ctx->stream : nullptr; }

// ---------------------------------------------------------------------------------------------
// batched independent replicas (extension: many cascades advanced by one graph launch)
// ---------------------------------------------------------------------------------------------
struct mg_batch {
    std::vector<mg_context *> ctxs;
    std::vector<uint64_t> gens;          // each context's generation when the graphs were captured
    int steps_per_launch = 1;
    cudaStream_t stream = nullptr;
    cudaGraphExec_t exec_k = nullptr;    // steps_per_launch loop bodies of every replica
    cudaGraphExec_t exec_1 = nullptr;    // one loop body of every replica (remainders)
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    std::vector<cudaEvent_t> ev_ctx;
    int launches_per_step = 0;
    std::string err;
};

namespace {

#define MB_CK(call)                                                                             \
    do {                                                                                        \
        cudaError_t e_ = (call);                                                                \
        if (e_ != cudaSuccess) {                                                                \
            b->err = std::string(#call) + ": " + cudaGetErrorString(e_);                       \
            return MG_ERR_CUDA;                                                                 \
        }                                                                                       \
    } while (0)

// Fork/join capture: every replica's stream joins the batch stream's capture, records `steps`
// loop bodies, and the batch stream joins them all at the end. The replicas share no memory, so
// the graph holds one independent branch per replica.
mg_status capture_batch(mg_batch *b, int steps, cudaGraphExec_t *exec, int *n_nodes) {
    cudaGraph_t graph = nullptr;
    MB_CK(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e = cudaEventRecord(b->ev_fork, b->stream);
    for (size_t r = 0; r < b->ctxs.size() && e == cudaSuccess; r++) {
        mg_context *ctx = b->ctxs[r];
        e = cudaStreamWaitEvent(ctx->stream, b->ev_fork, 0);
        for (int k = 0; k < steps && e == cudaSuccess; k++) {
            seq_step(ctx, nullptr);
            e = cudaGetLastError();
        }
        if (e == cudaSuccess) e = cudaEventRecord(b->ev_ctx[r], ctx->stream);
        if (e == cudaSuccess) e = cudaStreamWaitEvent(b->stream, b->ev_ctx[r], 0);
    }
    const cudaError_t e_end = cudaStreamEndCapture(b->stream, &graph);
    if (e != cudaSuccess || e_end != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        b->err = std::string("batch capture: ") + cudaGetErrorString(e != cudaSuccess ? e : e_end);
        return MG_ERR_CUDA;
    }
    size_t nn = 0;
    cudaGraphGetNodes(graph, nullptr, &nn);
    *n_nodes = static_cast<int>(nn);
    e = cudaGraphInstantiate(exec, graph, 0);
    cudaGraphDestroy(graph);
    if (e != cudaSuccess) { b->err = std::string("batch graph instantiate: ") + cudaGetErrorString(e); return MG_ERR_CUDA; }
    return MG_OK;
}

mg_status batch_capture_all(mg_batch *b) {
    if (b->exec_k) { cudaGraphExecDestroy(b->exec_k); b->exec_k = nullptr; }
    if (b->exec_1) { cudaGraphExecDestroy(b->exec_1); b->exec_1 = nullptr; }
    for (mg_context *ctx : b->ctxs) MB_CK(cudaStreamSynchronize(ctx->stream));
    int nk = 0, n1 = 0;
    mg_status st = capture_batch(b, b->steps_per_launch, &b->exec_k, &nk);
    if (st == MG_OK && b->steps_per_launch > 1) st = capture_batch(b, 1, &b->exec_1, &n1);
    if (st != MG_OK) return st;
    b->launches_per_step = b->steps_per_launch > 1 ? n1 : nk;
    for (size_t r = 0; r < b->ctxs.size(); r++) b->gens[r] = b->ctxs[r]->gen;
    return MG_OK;
}

}  // namespace

mg_status mg_batch_create(mg_context *const *ctxs, int32_t n, int32_t steps_per_launch, mg_batch **out) {
    if (!ctxs || n < 1 || !out || steps_per_launch < 1) return MG_ERR_ARG;
    for (int32_t r = 0; r < n; r++) {
        if (!ctxs[r]) return MG_ERR_ARG;
        for (int32_t q = 0; q < r; q++)
            if (ctxs[q] == ctxs[r]) { g_create_error = "mg_batch_create: a context appears twice"; return MG_ERR_ARG; }
        if (!ctxs[r]->prepared || !ctxs[r]->pot_ready) {
            g_create_error = "mg_batch_create: replica " + std::to_string(r) + " is not prepared";
            return MG_ERR_STATE;
        }
    }
    auto *b = new mg_batch();
    b->ctxs.assign(ctxs, ctxs + n);
    b->gens.assign(n, 0);
    b->steps_per_launch = steps_per_launch;
    b->ev_ctx.assign(n, nullptr);
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming);
    if (e == cudaSuccess) e = cudaEventCreateWithFlags(&b->ev_join, cudaEventDisableTiming);
    for (int32_t r = 0; r < n && e == cudaSuccess; r++) e = cudaEventCreateWithFlags(&b->ev_ctx[r], cudaEventDisableTiming);
    if (e != cudaSuccess) {
        g_create_error = std::string("mg_batch_create: ") + cudaGetErrorString(e);
        mg_batch_destroy(b);
        return MG_ERR_CUDA;
    }
    if (batch_capture_all(b) != MG_OK) {
        g_create_error = b->err;
        mg_batch_destroy(b);
        return MG_ERR_CUDA;
    }
    *out = b;
    return MG_OK;
}

mg_status mg_batch_run(mg_batch *b, int64_t nsteps, int32_t sync) {
    if (!b || nsteps < 0) return MG_ERR_ARG;
    for (size_t r = 0; r < b->ctxs.size(); r++) {
        if (!b->ctxs[r]->prepared) { b->err = "replica " + std::to_string(r) + " is not prepared"; return MG_ERR_STATE; }
        if (b->ctxs[r]->gen != b->gens[r]) {  // precision, tuning or potential changed since the capture
            mg_status st = batch_capture_all(b);
            if (st != MG_OK) return st;
            break;
        }
    }
    // the batch runs after each replica's pending work, and each replica's later work after the batch
    for (size_t r = 0; r < b->ctxs.size(); r++) {
        mg_context *ctx = b->ctxs[r];
        if (ctx->vmax_stale) {
            launch_vmax_full(ctx->lc(), ctx->g, ctx->s, ctx->in, ctx->d_sp);
            ctx->vmax_stale = false;
        }
        MB_CK(cudaEventRecord(b->ev_ctx[r], ctx->stream));
        MB_CK(cudaStreamWaitEvent(b->stream, b->ev_ctx[r], 0));
    }
    const int64_t k = b->steps_per_launch;
    for (int64_t i = 0; i < nsteps / k; i++) MB_CK(cudaGraphLaunch(b->exec_k, b->stream));
    for (int64_t i = 0; i < nsteps % k; i++) MB_CK(cudaGraphLaunch(b->exec_1, b->stream));
    MB_CK(cudaEventRecord(b->ev_join, b->stream));
    for (mg_context *ctx : b->ctxs) {
        MB_CK(cudaStreamWaitEvent(ctx->stream, b->ev_join, 0));
        ctx->energy_valid = false;
    }
    if (!sync) return MG_OK;
    MB_CK(cudaStreamSynchronize(b->stream));
    for (size_t r = 0; r < b->ctxs.size(); r++) {
        mg_context *ctx = b->ctxs[r];
        uint32_t bits = 0;
        mg_status st = read_device_errors(ctx, &bits);
        if (st == MG_OK) st = status_from_bits(ctx, bits);
        if (st != MG_OK) {
            b->err = "replica " + std::to_string(r) + ": " + ctx->err;
            return st;
        }
    }
    return MG_OK;
}

mg_status mg_batch_launches_per_step(const mg_batch *b, int32_t *n) {
    if (!b || !n) return MG_ERR_ARG;
    *n = b->launches_per_step;
    return MG_OK;
}

void *mg_batch_stream(const mg_batch *b) { return b ? (void *) b->stream : nullptr; }

const char *mg_batch_last_error(const mg_batch *b) { return b ? b->err.c_str() : g_create_error.c_str(); }

mg_status mg_batch_destroy(mg_batch *b) {
    if (!b) return MG_ERR_ARG;
    if (b->stream) cudaStreamSynchronize(b->stream);
    if (b->exec_k) cudaGraphExecDestroy(b->exec_k);
    if (b->exec_1) cudaGraphExecDestroy(b->exec_1);
    if (b->ev_fork) cudaEventDestroy(b->ev_fork);
    if (b->ev_join) cudaEventDestroy(b->ev_join);
    for (cudaEvent_t e : b->ev_ctx) if (e) cudaEventDestroy(e);
    if (b->stream) cudaStreamDestroy(b->stream);
    delete b;
    return MG_OK;
}

mg_status mg_host_register(void *ptr, uint64_t bytes) {
    if (!ptr || bytes == 0) return MG_ERR_ARG;
    cudaError_t e = cudaHostRegister(ptr, bytes, cudaHostRegisterDefault);
    if (e != cudaSuccess) { g_create_error = cudaGetErrorString(e); return MG_ERR_CUDA; }
    return MG_OK;
}
mg_status mg_host_unregister(void *ptr) {
    if (!ptr) return MG_ERR_ARG;
    cudaError_t e = cudaHostUnregister(ptr);
    if (e != cudaSuccess) { g_create_error = cudaGetErrorString(e); return MG_ERR_CUDA; }
    return MG_OK;
}

}  // extern "C"
