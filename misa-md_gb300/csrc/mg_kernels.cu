// GB300 (sm_103a) kernels for MISA-MD's per-step EAM hot path.
//
// Layout: structure-of-arrays over the reference's ghost-extended slot grid (doubled x), one thread
// per local slot. The lattice density and force passes are full-neighbour gathers over the offset
// table pruned to sites that can lie inside the cutoff (no Newton-3 scatter, no reverse fold, no
// atomics); inter atoms (few) keep the reference's structure for their own sums, and the lattice
// owners they touch gather their Newton-3 shares in a fixed order. The periodic ghost copy replaces
// the MPI halo exchange.
//
// Exact-rounding intrinsics (__dadd_rn / __dmul_rn / __ddiv_rn) are used wherever the reference's
// result must be reproduced bit for bit: velocity-Verlet, the decide distance test, the
// Wigner-Seitz mapping, ghost shifts and setv.

#include <algorithm>
#include <climits>
#include <cstddef>
#include <cstdio>

#include "mg_internal.h"

namespace mg {

// ------------------------------------------------------------------------------------------------
// constant tables
// ------------------------------------------------------------------------------------------------
__constant__ double c_mass[3];

void configure_manage_kernel();
void set_mass_table(cudaStream_t stream) {
    configure_manage_kernel();
    const double mass[3] = {atom_mass(0), atom_mass(1), atom_mass(2)};
    cudaMemcpyToSymbolAsync(c_mass, mass, sizeof(mass), 0, cudaMemcpyHostToDevice, stream);
    cudaStreamSynchronize(stream);
}

// ------------------------------------------------------------------------------------------------
// index helpers
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ int lin(const Geom &g, int x, int y, int z) { return (z * g.Sy + y) * g.Sx + x; }
// parity-split index of a slot (x even and odd sites in two halves) for the mixed form's gather arrays
__device__ __forceinline__ int sidx(const Geom &g, int s) { return (s & 1) * g.half + (s >> 1); }
// Thread order of the gathers. Warps always cover one site parity, so the candidate loop reads
// warp-uniform offsets. Order 0: all even local sites (k, j, i order), then all odd ones. Order 1:
// each run of 64 threads covers 32 consecutive even sites (first warp) and the 32 odd sites beside
// them (second warp), so both halves of each output sector are written close in time. The
// autotuner picks per kernel. Returns -1 past the end.
__device__ __forceinline__ int gather_site(const Geom &g, int t, int order, int &par, int &u) {
    if (order) {
        par = (t >> 5) & 1;
        u = ((t >> 6) << 5) | (t & 31);  // index among the sites of this parity
    } else {
        par = t >= g.n_local_half ? 1 : 0;
        u = par ? t - g.n_local_half : t;
    }
    if (u >= g.n_local_half) return -1;
    const int ih = u % g.nxh;
    const int r = u / g.nxh;
    return lin(g, 2 * ih + par + g.gx, r % g.by + g.gy, r / g.by + g.gz);
}
__device__ __forceinline__ int gather_slot(const Geom &g, int t, int order, int &par) {
    int u;
    return gather_site(g, t, order, par, u);
}
// threads to launch for the gathers
inline int gather_threads(const Geom &g, int order) {
    return order ? ((g.n_local_half + 31) / 32) * 64 : 2 * g.n_local_half;
}

__device__ __forceinline__ int local_slot(const Geom &g, int t, int &i, int &j, int &k) {
    i = t % g.bx;
    const int r = t / g.bx;
    j = r % g.by;
    k = r / g.by;
    return lin(g, i + g.gx, j + g.gy, k + g.gz);
}

// The slot a ghost (or local) slot mirrors under the periodic self-exchange, with the per-dimension
// shift the exchange adds (src/pack/lat_particle_packer.cpp:22-32: +L when sent LOWER, -L HIGHER).
__device__ __forceinline__ int wrap_axis(int c, int g, int b, int &sgn) {
    if (c < g) { sgn = -1; return c + b; }
    if (c >= g + b) { sgn = 1; return c - b; }
    sgn = 0;
    return c;
}
__device__ __forceinline__ int owner_slot(const Geom &g, int s) {
    const int X = s % g.Sx, r = s / g.Sx, Y = r % g.Sy, Z = r / g.Sy;
    int a, b, c;
    return lin(g, wrap_axis(X, g.gx, g.bx, a), wrap_axis(Y, g.gy, g.by, b), wrap_axis(Z, g.gz, g.bz, c));
}

// ------------------------------------------------------------------------------------------------
// Wigner-Seitz mapping (src/lattice/ws_utils.cpp:66-189), one rank: sub-box low corner at 0.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void voronoy_exact(double X, double Y, double Z, double lc, long long &cx, long long &cy,
                                              long long &cz) {
    const double qx = __ddiv_rn(X, lc), qy = __ddiv_rn(Y, lc), qz = __ddiv_rn(Z, lc);
    cx = llround(qx);
    cy = llround(qy);
    cz = llround(qz);
    const double dx = __dsub_rn(qx, (double) cx);
    const double dy = __dsub_rn(qy, (double) cy);
    const double dz = __dsub_rn(qz, (double) cz);
    const bool bx = dx > 0, by = dy > 0, bz = dz > 0;
    cx = 2 * cx;
    const double plane = __dadd_rn(__dadd_rn(__dadd_rn(bx ? dx : -dx, by ? dy : -dy), bz ? dz : -dz), -0.75);
    if (plane >= 0.0) {
        cx += bx ? 1 : -1;
        cy += by ? 0 : -1;
        cz += bz ? 0 : -1;
    }
}
// The integers above depend on the quotient q = RN(X / lc) only through three decisions per axis
// (the nearest integer, the sign of q minus it) and the sign of the bisector-plane sum. The quotient
// is first estimated as RN(X * RN(1 / lc)), within 3 * 2^-53 |q| of RN(X / lc), i.e. below 4e-10 for
// |q| < 2^20. Where every decision clears its boundary by kWsMargin, far above that error, the
// estimate makes the same decisions (the plane sum is the same monotone chain of rounded additions
// on inputs that moved by less than the margin), so the integers are the exact search's. Sites,
// half-way points, bisector planes, NaN and huge coordinates take the exact divisions. On this
// part an FP64 division costs several times a multiply, and the list manager runs these searches
// in a single block, so their latency is its own.
constexpr double kWsMargin = 1e-9;
__device__ __forceinline__ void voronoy(double X, double Y, double Z, const Geom &g, long long &cx, long long &cy,
                                        long long &cz) {
    const double qx = __dmul_rn(X, g.inv_a0), qy = __dmul_rn(Y, g.inv_a0), qz = __dmul_rn(Z, g.inv_a0);
    const double rx = rint(qx), ry = rint(qy), rz = rint(qz);
    const double dx = __dsub_rn(qx, rx), dy = __dsub_rn(qy, ry), dz = __dsub_rn(qz, rz);
    const double ax = fabs(dx), ay = fabs(dy), az = fabs(dz);
    const double plane = __dadd_rn(__dadd_rn(__dadd_rn(ax, ay), az), -0.75);
    const double amax = fmax(ax, fmax(ay, az)), amin = fmin(ax, fmin(ay, az));
    const double qmax = fmax(fabs(qx), fmax(fabs(qy), fabs(qz)));
    const bool clear = amin > kWsMargin && amax < 0.5 - kWsMargin && fabs(plane) > kWsMargin && qmax < 1048576.0;
    if (!clear) {
        voronoy_exact(X, Y, Z, g.a0, cx, cy, cz);
        return;
    }
    cx = 2 * (long long) rx;
    cy = (long long) ry;
    cz = (long long) rz;
    if (plane >= 0.0) {
        cx += dx > 0 ? 1 : -1;
        cy += dy > 0 ? 0 : -1;
        cz += dz > 0 ? 0 : -1;
    }
}
__device__ __forceinline__ uint32_t is_out_box(const Geom &g, double x, double y, double z) {
    long long cx, cy, cz;
    voronoy(x, y, z, g, cx, cy, cz);
    uint32_t f = kInBox;
    if (cx < 0) f |= kXLow; else if (cx >= g.bx) f |= kXHigh;
    if (cy < 0) f |= kYLow; else if (cy >= g.by) f |= kYHigh;
    if (cz < 0) f |= kZLow; else if (cz >= g.bz) f |= kZHigh;
    return f;
}
// ghost-extended coordinates of the nearest site (ws::getNearLatCoord)
__device__ __forceinline__ void near_lat_coord(const Geom &g, double x, double y, double z, long long c[3]) {
    voronoy(x, y, z, g, c[0], c[1], c[2]);
    c[0] += g.gx;
    c[1] += g.gy;
    c[2] += g.gz;
}
// ws::findNearLatIndexInSubBox: -1 outside the sub-box
__device__ __forceinline__ int near_index_in_sub_box(const Geom &g, double x, double y, double z) {
    long long cx, cy, cz;
    voronoy(x, y, z, g, cx, cy, cz);
    if (cx < 0 || cy < 0 || cz < 0 || cx >= g.bx || cy >= g.by || cz >= g.bz) return -1;
    return lin(g, (int) cx + g.gx, (int) cy + g.gy, (int) cz + g.gz);
}
// lattice site of a slot in global coordinates (decide's formula, src/atom.cpp:34-38, extended to
// ghost slots)
__device__ __forceinline__ void site_of(const Geom &g, int X, int Y, int Z, double &xs, double &ys, double &zs) {
    const int i = X - g.gx, j = Y - g.gy, k = Z - g.gz;
    const double half = (X & 1) ? 0.5 : 0.0;
    xs = __dmul_rn((double) i * 0.5, g.a0);
    ys = __dmul_rn((double) j + half, g.a0);
    zs = __dmul_rn((double) k + half, g.a0);
}
__device__ __forceinline__ float4 make_u4(const Geom &g, double x, double y, double z, double xs, double ys,
                                          double zs, int type) {
    return make_float4(__double2float_rn(__dmul_rn(__dsub_rn(x, xs), g.inv_h)),
                       __double2float_rn(__dmul_rn(__dsub_rn(y, ys), g.inv_h)),
                       __double2float_rn(__dmul_rn(__dsub_rn(z, zs), g.inv_h)), __int_as_float(type));
}

// u4 of a vacant slot: NaN coordinates, so every distance test against it fails without a type
// check in the candidate loops; w = INVALID
__device__ __forceinline__ float4 vacant_u4() {
    const float nan = __int_as_float(0x7fffffff);
    return make_float4(nan, nan, nan, __int_as_float(kInvalid));
}
// one 32-byte read-only load (sm_100 and later): a force record of the mixed form
__device__ __forceinline__ void ld_nc_v8(const float *p, float (&v)[8]) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(v[0]), "=f"(v[1]), "=f"(v[2]), "=f"(v[3]), "=f"(v[4]), "=f"(v[5]), "=f"(v[6]), "=f"(v[7])
        : "l"(p));
}
// Pairs of floats in one 64-bit register pair: sm_100 and later execute add/sub/mul/fma .f32x2 as
// one instruction, each lane rounded exactly as the scalar operation.
struct f2 {
    unsigned long long v;
};
__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 a, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(a.v));
}
__device__ __forceinline__ f2 f2_sub(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 f2_add(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 f2_mul(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r.v) : "l"(a.v), "l"(b.v));
    return r;
}
__device__ __forceinline__ f2 f2_fma(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(a.v), "l"(b.v), "l"(c.v));
    return r;
}
__device__ __forceinline__ double dt_inv_m_of(const StepParams *p, int type) {
    return type == 0 ? p->dt_inv_m[0] : (type == 1 ? p->dt_inv_m[1] : p->dt_inv_m[2]);
}
// |v|^2 in the order the oracle computes it ((vx^2 + vy^2) + vz^2, each operation rounded)
__device__ __forceinline__ double speed2(double vx, double vy, double vz) {
    return __dadd_rn(__dadd_rn(__dmul_rn(vx, vx), __dmul_rn(vy, vy)), __dmul_rn(vz, vz));
}
// The max-|v|^2 words feed only the variable-timestep rule; the kicks of a fixed-dt run skip them, and
// the host recomputes them (k_vmax_full) before the first step after the rule is switched on.
__device__ __forceinline__ bool variable_dt(const StepParams *sp) { return sp->dx_max > 0.0; }
// Max of v2 over the lanes that call this together, then one atomicMax per such group into a word
// picked by the warp's index, so the words see few atomics each. Non-negative doubles order like
// their bit patterns, so the max is taken on the 64-bit patterns, high word first.
__device__ __forceinline__ void note_vmax2(StepParams *sp, double v2) {
    const unsigned mask = __activemask();
    const unsigned long long b = (unsigned long long) __double_as_longlong(v2);
    const unsigned hi = (unsigned) (b >> 32), lo = (unsigned) b;
    const unsigned mhi = __reduce_max_sync(mask, hi);
    const unsigned mlo = __reduce_max_sync(mask, hi == mhi ? lo : 0u);
    if ((threadIdx.x & 31) == (unsigned) (__ffs(mask) - 1)) {
        const int w = (blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) & (kVmaxSlots - 1);
        atomicMax(&sp->vmax2[w], ((unsigned long long) mhi << 32) | mlo);
    }
}
__device__ __forceinline__ void set_error(Inter &in, uint32_t bit) { atomicOr((unsigned *) &in.cnt[CNT_ERRORS], bit); }
// Lattice passes can fuse df / the half-kick only when no other kernel adds density or force to
// lattice slots afterwards, i.e. when there are no inter atoms.
__device__ __forceinline__ bool lattice_only(const Inter &in) { return in.cnt[CNT_INTER] == 0; }
// Whether the lattice force pass may take the second half-kick of slot sl itself: always without inter
// atoms; with them, for every atom the density pass's inter-atom sweep did not list (no inter atom
// within the cutoff, so no inter-atom force is added later). The listed owners are kicked by the
// inter-atom force pass's owner gather once their force is complete.
__device__ __forceinline__ bool kick_in_lattice_pass(const Inter &in, int sl) {
    return lattice_only(in) || !((in.touch_bits[sl >> 5] >> (sl & 31)) & 1u);
}
// FP64 displacement test of atom::decide (src/atom.cpp:34-42) for a local slot
__device__ __forceinline__ bool displaced_fp64(const Geom &g, const Slots &s, int sl) {
    const int X = sl % g.Sx, r = sl / g.Sx, Y = r % g.Sy, Z = r / g.Sy;
    double xs, ys, zs;
    site_of(g, X, Y, Z, xs, ys, zs);
    const double ex = __dsub_rn(s.x[sl], xs), ey = __dsub_rn(s.y[sl], ys), ez = __dsub_rn(s.z[sl], zs);
    double dist = __dmul_rn(ex, ex);
    dist = __dadd_rn(dist, __dmul_rn(ey, ey));
    dist = __dadd_rn(dist, __dmul_rn(ez, ez));
    return dist > g.thr;
}

// ------------------------------------------------------------------------------------------------
// spline evaluation
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ void locate_d(double x, double inv, int n, int &m, double &p) {
    p = x * inv;
    m = (int) p;
    m = max(0, min(m, n - 2));
    p -= m;
    p = fmin(p, 1.0);
}
__device__ __forceinline__ double val_d(const Knot64 *t, int m, double p) {
    const double2 *q = reinterpret_cast<const double2 *>(t + m);
    const double2 lo = __ldg(q), hi = __ldg(q + 1);  // {c0, c1}, {c2, c3}
    return fma(fma(fma(hi.y, p, hi.x), p, lo.y), p, lo.x);
}
__device__ __forceinline__ double der_d(const Knot64 *t, int m, double p) {
    const double2 *q = reinterpret_cast<const double2 *>(t + m);
    const double2 lo = __ldg(q), hi = __ldg(q + 1);  // {d0, d1}, {d2, 0}
    return fma(fma(hi.x, p, lo.y), p, lo.x);
}
__device__ __forceinline__ void locate_f(float x, float inv, int n, int &m, float &p) {
    p = x * inv;
    m = (int) p;
    m = max(0, min(m, n - 2));
    p -= (float) m;
    p = fminf(p, 1.0f);
}
// knot of a pair distance in the FP32 gathers: 0 < r < rc <= (nr - 1) dr, so only a guard against
// rounding at r ~ rc is needed (it keeps m on the last knot, whose record exists)
__device__ __forceinline__ void locate_r_f(float x, float inv, int n, int &m, float &p) {
    p = x * inv;
    m = min((int) p, n - 1);
    p -= (float) m;
}
__device__ __forceinline__ float val_f(const float4 *t, int m, float p) {
    const float4 c = __ldg(t + m);
    return fmaf(fmaf(fmaf(c.w, p, c.z), p, c.y), p, c.x);
}
__device__ __forceinline__ float der_f(const float4 *t, int m, float p) {
    const float4 c = __ldg(t + m);
    return fmaf(fmaf(c.z, p, c.y), p, c.x);
}
__device__ __forceinline__ void kahan(float &sum, float &comp, float term) {
    const float y = term - comp;
    const float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

// ------------------------------------------------------------------------------------------------
// AoS <-> SoA (the reference's AtomElement array crosses the boundary as raw records)
// ------------------------------------------------------------------------------------------------
__global__ void k_unpack_aos(Geom g, const mg_atom_element *aos, Slots s, Inter in, int types_ok_mask, bool mixed, int s0,
                             int s1) {
    const int t = s0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= s1) return;
    mg_atom_element a = aos[t];
    if (a.type < -1 || a.type > 2 || (a.type >= 0 && !((types_ok_mask >> a.type) & 1))) {
        set_error(in, MG_DEVERR_BAD_TYPE);
        a.type = kInvalid;
    }
    s.x[t] = a.x[0]; s.y[t] = a.x[1]; s.z[t] = a.x[2];
    s.vx[t] = a.v[0]; s.vy[t] = a.v[1]; s.vz[t] = a.v[2];
    s.fx[t] = a.f[0]; s.fy[t] = a.f[1]; s.fz[t] = a.f[2];
    s.rho[t] = a.rho; s.df[t] = a.df;
    s.type[t] = (int8_t) a.type;
    s.id[t] = a.id;
    {  // u4 in both precisions: the gathers' FP32 candidate test reads it
        const int X = t % g.Sx, r = t / g.Sx, Y = r % g.Sy, Z = r / g.Sy;
        double xs, ys, zs;
        site_of(g, X, Y, Z, xs, ys, zs);
        s.u4[sidx(g, t)] = a.type < 0 ? vacant_u4() : make_u4(g, a.x[0], a.x[1], a.x[2], xs, ys, zs, a.type);
    }
    if (mixed) s.df32[sidx(g, t)] = (float) a.df;
}

__global__ void k_pack_aos(Geom g, mg_atom_element *aos, Slots s, int fields, bool mixed, int s0, int s1) {
    const int t = s0 + blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= s1) return;
    mg_atom_element &a = aos[t];
    const double df = mixed ? (double) s.df32[sidx(g, t)] : s.df[t];
    if (fields == PACK_ALL) {
        mg_atom_element b;
        b.id = s.id[t];
        b.type = s.type[t];
        b.pad_ = 0;
        b.x[0] = s.x[t]; b.x[1] = s.y[t]; b.x[2] = s.z[t];
        b.v[0] = s.vx[t]; b.v[1] = s.vy[t]; b.v[2] = s.vz[t];
        b.f[0] = s.fx[t]; b.f[1] = s.fy[t]; b.f[2] = s.fz[t];
        b.rho = s.rho[t];
        b.df = df;
        a = b;
        return;
    }
    if (fields & PACK_RHO) a.rho = s.rho[t];
    if (fields & PACK_DF) a.df = df;
    if (fields & PACK_F) { a.f[0] = s.fx[t]; a.f[1] = s.fy[t]; a.f[2] = s.fz[t]; }
}

void launch_unpack_aos(const LaunchCtx &lc, const Geom &g, const mg_atom_element *aos, Slots s, Inter in,
                       int types_ok_mask, bool mixed, int s0, int s1) {
    if (s1 < 0) s1 = g.n_slots;
    if (s1 <= s0) return;
    const int b = 256;
    k_unpack_aos<<<(s1 - s0 + b - 1) / b, b, 0, lc.stream>>>(g, aos, s, in, types_ok_mask, mixed, s0, s1);
    launch_skin_dirty(lc, s);
}
__global__ void k_set_counts(Inter in, int n_inter) {
    in.cnt[CNT_INTER] = n_inter;
    in.cnt[CNT_GHOST] = 0;
    in.cnt[CNT_DISPLACED] = 0;
    in.cnt[CNT_DISP_RAW] = 0;
    *in.n_bucket = 0;
}
void launch_set_counts(const LaunchCtx &lc, Inter in, int n_inter) { k_set_counts<<<1, 1, 0, lc.stream>>>(in, n_inter); }
void launch_pack_aos(const LaunchCtx &lc, const Geom &g, mg_atom_element *aos, Slots s, int fields, bool mixed, int s0,
                     int s1) {
    if (s1 < 0) s1 = g.n_slots;
    if (s1 <= s0) return;
    const int b = 256;
    k_pack_aos<<<(s1 - s0 + b - 1) / b, b, 0, lc.stream>>>(g, aos, s, fields, mixed, s0, s1);
}

// ------------------------------------------------------------------------------------------------
// velocity-Verlet first half + drift (src/newton_motion.cpp:30-44) fused with the displacement test
// of atom::decide (src/atom.cpp:27-53). Displaced slots are collected unordered; the list kernel
// sorts them into the reference's k, j, i scan order.
// ------------------------------------------------------------------------------------------------
__global__ void k_site_table(double a0, int n, double *out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m < n) out[m] = __dmul_rn((double) m * 0.5, a0);  // site_of: (i * 0.5) * a0, (j + half) * a0
}
void launch_site_table(const LaunchCtx &lc, const Geom &g, double *site_half) {
    k_site_table<<<(g.n_site_half + 255) / 256, 256, 0, lc.stream>>>(g.a0, g.n_site_half, site_half);
}

// Displaced slots are recorded in scan order without a sort: firststep writes one byte per local slot
// (byte t for local index t, in k, j, i order; 1 = displaced). A count kernel sums the bytes of each
// group of kFirstThreads slots, a one-block scan turns the sums into offsets, and a collect kernel
// writes the slots in order. firststep keeps its early exits and needs no warp or block collective.
// decide's distance test (src/atom.cpp:34-42) with each operation rounded on its own; a displaced
// atom also counts itself into CNT_DISP_RAW, so the collection kernels can skip steps without any
// displaced atom.
__device__ __noinline__ bool exact_displaced(double ex, double ey, double ez, double thr, int *raw_count) {
    double dist = __dmul_rn(ex, ex);
    dist = __dadd_rn(dist, __dmul_rn(ey, ey));
    dist = __dadd_rn(dist, __dmul_rn(ez, ez));
    const bool d = dist > thr;
    if (d) atomicAdd(raw_count, 1);
    return d;
}

// the step's largest change of a displacement record: one reduction per group of converged lanes and
// one atomic max per group, spread over kSkinSlots words (squares of non-negative floats order like
// their bit patterns; a NaN orders above every number, so it forces a rebuild)
__device__ __forceinline__ void skin_note(const Slots &s, float d2) {
    const unsigned m = __activemask();
    const unsigned v = __reduce_max_sync(m, __float_as_uint(d2));
    if ((int) (threadIdx.x & 31) == __ffs(m) - 1) atomicMax(&s.skin->step_max2[blockIdx.x & (kSkinSlots - 1)], v);
}

// NewtonMotion::firststep for one lattice atom (src/newton_motion.cpp:30-55) and decide's displacement
// test (src/atom.cpp:34-42): v += c f, x += dt v (each operation rounded as the reference rounds it),
// the displacement record u4 (written to u4_out, parity-split index) and the displaced flag of local
// index t. MOVE = false: the test alone, on the current positions. u4_prev holds the record the last
// density pass read (for the skin's displacement bound).
template <bool MOVE, bool DECIDE>
__device__ __forceinline__ void first_half(const Geom &g, const Slots &s, const Inter &in, const StepParams *__restrict__ p,
                                           int sl, int t, int i, int j, int k, int ty, double vx, double vy, double vz,
                                           double fx, double fy, double fz, float4 *u4_out, const float4 *u4_prev) {
    double x = s.x[sl], y = s.y[sl], z = s.z[sl];
    if (MOVE) {
        const double c = dt_inv_m_of(p, ty);
        vx = __dadd_rn(vx, __dmul_rn(c, fx));
        vy = __dadd_rn(vy, __dmul_rn(c, fy));
        vz = __dadd_rn(vz, __dmul_rn(c, fz));
        const double dt = p->dt;
        x = __dadd_rn(x, __dmul_rn(dt, vx));
        y = __dadd_rn(y, __dmul_rn(dt, vy));
        z = __dadd_rn(z, __dmul_rn(dt, vz));
        s.vx[sl] = vx; s.vy[sl] = vy; s.vz[sl] = vz;
        s.x[sl] = x; s.y[sl] = y; s.z[sl] = z;
    }
    // the site from the table (the same rounded values site_of computes; gx is even, so the x parity
    // of the slot is i & 1)
    const int par = i & 1;
    const double xs = g.site_half[i], ys = g.site_half[2 * j + par], zs = g.site_half[2 * k + par];
    const double ex = __dsub_rn(x, xs), ey = __dsub_rn(y, ys), ez = __dsub_rn(z, zs);
    const float exf = __double2float_rn(ex), eyf = __double2float_rn(ey), ezf = __double2float_rn(ez);
    if (MOVE) {
        const float ih = g.inv_h_f;
        const float4 nu = make_float4(exf * ih, eyf * ih, ezf * ih, __int_as_float(ty));
        const int si = sidx(g, sl);
        if (g.skin_h > 0.f) {  // read before the store: in place, u4_prev is u4_out
            const float4 o = u4_prev[si];
            const float dx = nu.x - o.x, dy = nu.y - o.y, dz = nu.z - o.z;
            skin_note(s, dx * dx + dy * dy + dz * dz);
        }
        u4_out[si] = nu;
    }
    if (DECIDE) {
        // the exact FP64 test of decide runs only where the FP32 distance is not clearly below it
        // (a call, so the rare path stays a branch instead of being evaluated for every atom)
        const bool disp = !(exf * exf + eyf * eyf + ezf * ezf < g.thr_lo_f) &&
                          exact_displaced(ex, ey, ez, g.thr, &in.cnt[CNT_DISP_RAW]);
        in.dflag[t] = disp ? 1 : 0;
    }
}

// fused: the previous step's force pass already took this firststep for every local slot and wrote
// its displacement records into this step's u4 buffer (when no inter atoms exist; else the work is
// done here). Every local slot's u4 is written, vacancies included, so the two buffers a fused graph
// alternates between are always complete.
// alt: inside a graph whose bodies alternate their u4 buffers, where the previous body's records are
// in s.u4n
// A grid-stride loop over a grid of a few blocks per SM: a fused body's launch, which returns at once,
// then costs one small launch instead of a grid over every slot.
template <bool MOVE, bool DECIDE>
__global__ void __launch_bounds__(kFirstThreads) k_firststep(Geom g, Slots s, Inter in, const StepParams *__restrict__ p,
                                                             int t0, int t1, bool fused, bool alt) {
    if (fused && lattice_only(in)) return;
    for (int t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
        int i, j, k;
        const int sl = local_slot(g, t, i, j, k);
        const int ty = s.type[sl];
        if (ty < 0) {
            if (DECIDE) in.dflag[t] = 0;
            if (MOVE) s.u4[sidx(g, sl)] = vacant_u4();
            continue;
        }
        if (MOVE)
            first_half<true, DECIDE>(g, s, in, p, sl, t, i, j, k, ty, s.vx[sl], s.vy[sl], s.vz[sl], s.fx[sl], s.fy[sl],
                                     s.fz[sl], s.u4, alt ? s.u4n : s.u4);
        else
            first_half<false, DECIDE>(g, s, in, p, sl, t, i, j, k, ty, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, s.u4, s.u4);
    }
}

// one warp per group of kFirstThreads flag bytes (8 per lane, read as one 64-bit word): its count
__global__ void k_disp_count(Inter in, int nblocks) {
    if (in.cnt[CNT_DISP_RAW] == 0) return;  // nothing displaced this step (the usual case)
    const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (b >= nblocks) return;
    const unsigned long long w = reinterpret_cast<const unsigned long long *>(in.dflag)[b * 32 + (threadIdx.x & 31)];
    int c = __popcll(w);  // bytes are 0 or 1
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if ((threadIdx.x & 31) == 0) in.dblock[b] = c;
}

// one block: counts a[0..n) -> base + exclusive offsets (in place); returns base + the total (every
// thread). Each thread takes one contiguous chunk: a pass summing it, one block scan of the chunk
// sums, and a pass writing the chunk's offsets (one scan instead of one per blockDim.x counts).
__device__ int block_scan_counts(int *a, int n, int base) {
    __shared__ int warp_tot[32];
    const int per = (n + (int) blockDim.x - 1) / (int) blockDim.x;
    const int b0 = min(n, (int) threadIdx.x * per), b1 = min(n, b0 + per);
    int v = 0;
#pragma unroll 4
    for (int b = b0; b < b1; b++) v += a[b];
    int x = v;  // inclusive warp scan of the chunk sums
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) >= o) x += y;
    }
    if ((threadIdx.x & 31) == 31) warp_tot[threadIdx.x >> 5] = x;
    __syncthreads();
    if (threadIdx.x < 32) {
        int w = threadIdx.x < (blockDim.x >> 5) ? warp_tot[threadIdx.x] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (threadIdx.x >= o) w += y;
        }
        warp_tot[threadIdx.x] = w;  // inclusive over warps
    }
    __syncthreads();
    int run = base + ((threadIdx.x >> 5) ? warp_tot[(threadIdx.x >> 5) - 1] : 0) + x - v;
    for (int b = b0; b < b1; b++) {
        const int c = a[b];
        a[b] = run;
        run += c;
    }
    const int total = base + warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();  // warp_tot is free again for a later call
    return total;
}

// one block: block counts -> exclusive offsets (in place), total -> CNT_DISPLACED (clamped to dcap)
__global__ void __launch_bounds__(1024) k_disp_scan(Inter in, int nblocks) {
    if (in.cnt[CNT_DISP_RAW] == 0) {  // nothing displaced this step (the usual case)
        if (threadIdx.x == 0) in.cnt[CNT_DISPLACED] = 0;
        return;
    }
    int total = block_scan_counts(in.dblock, nblocks, 0);
    if (threadIdx.x == 0) {
        if (total > in.dcap) { set_error(in, MG_DEVERR_DISPLACED_OVERFLOW); total = in.dcap; }
        in.cnt[CNT_DISPLACED] = total;
        in.cnt[CNT_DISP_RAW] = 0;
    }
}

// one warp per group of kFirstThreads flag bytes: its displaced slots, in order, at the group's offset
__global__ void k_disp_collect(Geom g, Inter in, int nblocks) {
    if (in.cnt[CNT_DISPLACED] == 0) return;
    const int b = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    if (b >= nblocks) return;
    const int lane = threadIdx.x & 31;
    unsigned long long w = reinterpret_cast<const unsigned long long *>(in.dflag)[b * 32 + lane];
    const int c = __popcll(w);
    int incl = c;  // inclusive scan over the lanes
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (c == 0) return;
    int rank = in.dblock[b] + incl - c;
    for (int byte = 0; w; byte++, w >>= 8) {
        if ((w & 0xff) == 0) continue;
        if (rank < in.dcap) {
            int i, j, k;
            in.displaced[rank] = local_slot(g, b * kFirstThreads + lane * 8 + byte, i, j, k);
        }
        rank++;
    }
}

void launch_firststep(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, const StepParams *p, bool decide, int t0,
                      int t1, bool fused, bool alt) {
    if (t1 < 0) t1 = g.n_local;
    if (t1 <= t0) return;
    const int b = kFirstThreads, n = std::min((t1 - t0 + b - 1) / b, lc.num_sms * 8);
    if (decide) k_firststep<true, true><<<n, b, 0, lc.stream>>>(g, s, in, p, t0, t1, fused, alt);
    else k_firststep<true, false><<<n, b, 0, lc.stream>>>(g, s, in, p, t0, t1, fused, alt);
}
void launch_decide_scan(const LaunchCtx &lc, const Geom &g, Slots s, Inter in) {
    const int b = kFirstThreads, n = std::min((g.n_local + b - 1) / b, lc.num_sms * 8);
    k_firststep<false, true><<<n, b, 0, lc.stream>>>(g, s, in, nullptr, 0, g.n_local, false, false);
}
void launch_displaced_collect(const LaunchCtx &lc, const Geom &g, Inter in) {
    const int nblocks = (g.n_local + kFirstThreads - 1) / kFirstThreads;
    const int grid = (nblocks + 7) / 8;  // 8 warps (groups) per 256-thread block
    k_disp_count<<<grid, 256, 0, lc.stream>>>(in, nblocks);
    k_disp_scan<<<1, 1024, 0, lc.stream>>>(in, nblocks);
    k_disp_collect<<<grid, 256, 0, lc.stream>>>(g, in, nblocks);
}

__global__ void k_inter_firststep(Inter in, const StepParams *__restrict__ p) {
    const int n = in.cnt[CNT_INTER];
    const double dt = p->dt;
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x) {
        const double c = dt_inv_m_of(p, in.type[a]);
        double vx = __dadd_rn(in.vx[a], __dmul_rn(c, in.fx[a]));
        double vy = __dadd_rn(in.vy[a], __dmul_rn(c, in.fy[a]));
        double vz = __dadd_rn(in.vz[a], __dmul_rn(c, in.fz[a]));
        in.vx[a] = vx; in.vy[a] = vy; in.vz[a] = vz;
        in.x[a] = __dadd_rn(in.x[a], __dmul_rn(dt, vx));
        in.y[a] = __dadd_rn(in.y[a], __dmul_rn(dt, vy));
        in.z[a] = __dadd_rn(in.z[a], __dmul_rn(dt, vz));
    }
}
void launch_inter_firststep(const LaunchCtx &lc, Inter in, const StepParams *p) {
    k_inter_firststep<<<lc.num_sms, 256, 0, lc.stream>>>(in, p);
}

// ------------------------------------------------------------------------------------------------
// periodic ghost copy (replaces AtomList::exchangeAtom + LatPacker, src/atom/atom_list.cpp:51-57):
// ghost slot <- (type, x with per-dimension +-L) of its owner. One hop reproduces the reference's
// x -> y -> z phases exactly: each coordinate receives at most one shift.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ int ghost_slot(const Geom &g, int t) {
    const int nz = 2 * g.gz * g.Sy * g.Sx;
    const int ny = 2 * g.gy * g.bz * g.Sx;
    int X, Y, Z;
    if (t < nz) {
        const int plane = g.Sy * g.Sx;
        int zz = t / plane;
        const int r = t % plane;
        Z = zz < g.gz ? zz : zz + g.bz;
        Y = r / g.Sx;
        X = r % g.Sx;
    } else if (t < nz + ny) {
        const int u = t - nz;
        const int row = g.Sx;
        const int yy = u / (g.bz * row);
        const int r = u % (g.bz * row);
        Y = yy < g.gy ? yy : yy + g.by;
        Z = g.gz + r / row;
        X = r % row;
    } else {
        const int u = t - nz - ny;
        const int xx = u % (2 * g.gx);
        const int r = u / (2 * g.gx);
        X = xx < g.gx ? xx : xx + g.bx;
        Y = g.gy + r % g.by;
        Z = g.gz + r / g.by;
    }
    return lin(g, X, Y, Z);
}

__device__ __forceinline__ void ghost_copy_one(const Geom &g, const Slots &s, int gs) {
    const int X = gs % g.Sx, r = gs / g.Sx, Y = r % g.Sy, Z = r / g.Sy;
    int sx, sy, sz;
    const int os = lin(g, wrap_axis(X, g.gx, g.bx, sx), wrap_axis(Y, g.gy, g.by, sy), wrap_axis(Z, g.gz, g.bz, sz));
    s.type[gs] = s.type[os];
    const double ox = s.x[os], oy = s.y[os], oz = s.z[os];
    s.x[gs] = sx ? __dadd_rn(ox, sx > 0 ? g.L[0] : -g.L[0]) : ox;
    s.y[gs] = sy ? __dadd_rn(oy, sy > 0 ? g.L[1] : -g.L[1]) : oy;
    s.z[gs] = sz ? __dadd_rn(oz, sz > 0 ? g.L[2] : -g.L[2]) : oz;
    s.u4[sidx(g, gs)] = s.u4[sidx(g, os)];
}
__global__ void k_ghost_copy(Geom g, Slots s) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n_ghost_slots) return;
    ghost_copy_one(g, s, ghost_slot(g, t));
}
void launch_ghost_copy(const LaunchCtx &lc, const Geom &g, Slots s, bool) {
    const int b = 256, n = (g.n_ghost_slots + b - 1) / b;
    k_ghost_copy<<<n, b, 0, lc.stream>>>(g, s);
}
// The ghost slots inside the local planes [k0, k1) (y-ghost rows, then x-ghost columns of each plane;
// their owners lie in the same plane), or (k0 < 0) the ghost planes below and above the box, whose
// owners are the top and bottom local planes. Together the calls cover every ghost slot once.
__global__ void k_ghost_copy_planes(Geom g, Slots s, int k0, int k1) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 < 0) {
        if (t < 2 * g.gz * g.Sy * g.Sx) ghost_copy_one(g, s, ghost_slot(g, t));  // the z-ghost planes come first
        return;
    }
    const int rows = 2 * g.gy * g.Sx, per = rows + 2 * g.gx * g.by;
    if (t >= (k1 - k0) * per) return;
    const int Z = g.gz + k0 + t / per, v = t % per;
    int X, Y;
    if (v < rows) {
        const int yy = v / g.Sx;
        Y = yy < g.gy ? yy : yy + g.by;
        X = v % g.Sx;
    } else {
        const int w = v - rows, xx = w % (2 * g.gx);
        X = xx < g.gx ? xx : xx + g.bx;
        Y = g.gy + w / (2 * g.gx);
    }
    ghost_copy_one(g, s, lin(g, X, Y, Z));
}
void launch_ghost_copy_planes(const LaunchCtx &lc, const Geom &g, Slots s, int k0, int k1) {
    const int b = 256;
    const int work = k0 < 0 ? 2 * g.gz * g.Sy * g.Sx : (k1 - k0) * (2 * g.gy * g.Sx + 2 * g.gx * g.by);
    if (work <= 0) return;
    k_ghost_copy_planes<<<(work + b - 1) / b, b, 0, lc.stream>>>(g, s, k0, k1);
}

// forward df (DfEmbedPacker, src/pack/df_embed_packer.cpp): lattice ghosts and ghost inter atoms
template <bool MIXED>
__global__ void k_ghost_df(Geom g, Slots s, Inter in) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < g.n_ghost_slots) {
        const int gs = ghost_slot(g, t);
        const int os = owner_slot(g, gs);
        if (MIXED) s.df32[sidx(g, gs)] = s.df32[sidx(g, os)];
        else s.df[gs] = s.df[os];
    }
    const int ng = in.cnt[CNT_GHOST];
    for (int q = t; q < ng; q += gridDim.x * blockDim.x) in.gdf[q] = in.df[in.groot[q]];
}
void launch_ghost_df(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, bool mixed) {
    const int b = 256, n = (g.n_ghost_slots + b - 1) / b;
    if (mixed) k_ghost_df<true><<<n, b, 0, lc.stream>>>(g, s, in);
    else k_ghost_df<false><<<n, b, 0, lc.stream>>>(g, s, in);
}
// the same copy for the ghost slots inside the local planes [k0, k1) (y-ghost rows, then x-ghost
// columns of each plane; their owners lie in the same plane), or (k0 < 0) for the ghost planes below
// and above the box together with the ghost inter atoms
template <bool MIXED>
__global__ void k_ghost_df_planes(Geom g, Slots s, Inter in, int k0, int k1) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (k0 < 0) {
        if (t < 2 * g.gz * g.Sy * g.Sx) {
            const int gs = ghost_slot(g, t);  // the z-ghost planes come first in the ghost enumeration
            const int os = owner_slot(g, gs);
            if (MIXED) s.df32[sidx(g, gs)] = s.df32[sidx(g, os)];
            else s.df[gs] = s.df[os];
        }
        const int ng = in.cnt[CNT_GHOST];
        for (int q = t; q < ng; q += gridDim.x * blockDim.x) in.gdf[q] = in.df[in.groot[q]];
        return;
    }
    const int rows = 2 * g.gy * g.Sx, per = rows + 2 * g.gx * g.by;
    if (t >= (k1 - k0) * per) return;
    const int Z = g.gz + k0 + t / per, v = t % per;
    int X, Y;
    if (v < rows) {
        const int yy = v / g.Sx;
        Y = yy < g.gy ? yy : yy + g.by;
        X = v % g.Sx;
    } else {
        const int w = v - rows, xx = w % (2 * g.gx);
        X = xx < g.gx ? xx : xx + g.bx;
        Y = g.gy + w / (2 * g.gx);
    }
    const int gs = lin(g, X, Y, Z);
    const int os = owner_slot(g, gs);
    if (MIXED) s.df32[sidx(g, gs)] = s.df32[sidx(g, os)];
    else s.df[gs] = s.df[os];
}
void launch_ghost_df_planes(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, bool mixed, int k0, int k1) {
    const int b = 256;
    const int work = k0 < 0 ? 2 * g.gz * g.Sy * g.Sx : (k1 - k0) * (2 * g.gy * g.Sx + 2 * g.gx * g.by);
    if (work <= 0) return;
    const int n = (work + b - 1) / b;
    if (mixed) k_ghost_df_planes<true><<<n, b, 0, lc.stream>>>(g, s, in, k0, k1);
    else k_ghost_df_planes<false><<<n, b, 0, lc.stream>>>(g, s, in, k0, k1);
}

// ------------------------------------------------------------------------------------------------
// lattice density pass (atom::latRho, src/atom.cpp:151-192, as a full gather) with dF/drho fused
// when no inter or far atom adds density afterwards (atom::latDf, src/atom.cpp:286-309).
// Warps are parity-uniform (gather_slot), so the candidate loop reads warp-uniform constants; far
// atoms continue over the entries beyond the pruned set.
// ------------------------------------------------------------------------------------------------
// FP32 candidate test of the FP64 gathers: r^2 from the u4 displacements, against rc^2 (1 + 1e-4).
// Its error is below 1e-6 of rc^2, so every pair the exact FP64 test accepts passes it; vacancies
// (NaN) never do. Only candidates that pass load their FP64 positions.
__device__ __forceinline__ bool near_f32(const Geom &g, f2 uixy, float uiz, float4 D, float4 uj) {
    const f2 dxy = f2_sub(f2_sub(uixy, f2_pack(uj.x, uj.y)), f2_pack(D.x, D.y));
    const float dz = (uiz - uj.z) - D.z;
    float dx, dy;
    f2_unpack(dxy, dx, dy);
    return dx * dx + dy * dy + dz * dz < g.rc2_pre;
}

template <int PAR>
__device__ __forceinline__ double rho_sum_fp64(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt, int sl,
                                               int si, float4 ui, double xi, double yi, double zi, int q0, int q1) {
    double acc = 0.0;
    const f2 uixy = f2_pack(ui.x, ui.y);
#pragma unroll 4
    for (int q = q0; q < q1; q++) {
        const float4 D = nt.cand[PAR][q];
        const float4 uj = __ldg(s.u4 + si + __float_as_int(D.w));
        if (!near_f32(g, uixy, ui.z, D, uj)) continue;
        const int sj = sl + nt.lat[PAR][q];
        const int tj = __float_as_int(uj.w);
        const double dx = xi - s.x[sj], dy = yi - s.y[sj], dz = zi - s.z[sj];
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < g.rc2) {
            const double r = r2 * rsqrt(r2);
            int m; double p;
            locate_d(r, pt.inv_dr, pt.nr, m, p);
            acc += val_d(pt.rho_v + tj * pt.nr, m, p);
        }
    }
    return acc;
}

__device__ __forceinline__ void k_lat_rho_fp64_site(int t, const NeighTables &nt, const Geom &g, const Slots &s, const Inter &in, const PotTables &pt, bool hook, int order) {
    int par;
    const int sl = gather_slot(g, t, order, par);
    if (sl < 0) return;
    const int ti = s.type[sl];
    if (ti < 0) { s.rho[sl] = 0.0; return; }
    const double xi = s.x[sl], yi = s.y[sl], zi = s.z[sl];
    const int si = sidx(g, sl);
    const float4 ui = s.u4[si];
    const int np = nt.npruned;
    double acc = par ? rho_sum_fp64<1>(nt, g, s, pt, sl, si, ui, xi, yi, zi, 0, np)
                     : rho_sum_fp64<0>(nt, g, s, pt, sl, si, ui, xi, yi, zi, 0, np);
    if (in.far_flag[sl]) {
        const int nf = nt.nfull;
        acc += par ? rho_sum_fp64<1>(nt, g, s, pt, sl, si, ui, xi, yi, zi, np, nf)
                   : rho_sum_fp64<0>(nt, g, s, pt, sl, si, ui, xi, yi, zi, np, nf);
    }
    s.rho[sl] = acc;
    if (!hook && lattice_only(in)) {
        int m; double p;
        locate_d(acc, pt.inv_drho, pt.nrho, m, p);
        s.df[sl] = der_d(pt.F_d + ti * pt.nrho, m, p);
    }
}
template <bool LOOP>  // LOOP: several sites per thread, one grid stride apart
__global__ void __launch_bounds__(512) k_lat_rho_fp64(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, PotTables pt, bool hook, int order, int tbase,
                                                       int nthreads) {
    const int t0 = tbase + blockIdx.x * blockDim.x + threadIdx.x;  // threads [tbase, nthreads)
    if (!LOOP) {
        if (t0 < nthreads) k_lat_rho_fp64_site(t0, nt, g, s, in, pt, hook, order);
        return;
    }
    for (int t = t0; t < nthreads; t += gridDim.x * blockDim.x) k_lat_rho_fp64_site(t, nt, g, s, in, pt, hook, order);
}

// r^2 of a candidate pair in half-lattice units (and the pair vector), each operation rounded as
// written: the density and force passes both compute it and must agree bit for bit on which pairs
// lie inside the cutoff (the force pass skips the tail candidates no site of a group had inside)
__device__ __forceinline__ float pair_r2(f2 uixy, float uiz, float4 D, float4 uj, f2 &dxy, float &dz) {
    dxy = f2_sub(f2_sub(uixy, f2_pack(uj.x, uj.y)), f2_pack(D.x, D.y));
    dz = __fsub_rn(__fsub_rn(uiz, uj.z), D.z);
    float dx, dy;
    f2_unpack(dxy, dx, dy);
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}
// one density term (in range): rho_tj(r)
__device__ __forceinline__ void rho_pair(const PotTables &pt, float r2, float4 uj, float &sum, float &comp) {
    const int tj = __float_as_int(uj.w);
    const float rp = r2 * rsqrtf(r2);
    int m; float p;
    locate_r_f(rp, pt.h_inv_dr_f, pt.nr, m, p);
    kahan(sum, comp, val_f(pt.rho_vf + tj * pt.nr, m, p));
}
template <int PAR>
__device__ __forceinline__ void rho_sum_mixed(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt, int si, float4 ui,
                                              int q0, int q1, float &sum, float &comp) {
    const float rc2 = g.rc2_h;
    const f2 uixy = f2_pack(ui.x, ui.y);
#pragma unroll 2  // 1, 4 and 8 measured slower
    for (int q = q0; q < q1; q++) {
        const float4 D = nt.cand[PAR][q];
        const float4 uj = __ldg(s.u4 + si + __float_as_int(D.w));
        f2 dxy; float dz;
        const float r2 = pair_r2(uixy, ui.z, D, uj, dxy, dz);
        if (r2 < rc2) rho_pair(pt, r2, uj, sum, comp);  // false for vacancies (NaN coordinates)
    }
}
// The pruned candidates [q0, q1), q1 - q0 <= 32, noting which this site has within rc + skin (bit j:
// candidate q0 + j; rcs2_h >= rc2_h). FULL: q1 - q0 is 32, known at compile time (the full chunks; a
// runtime count there costs registers).
template <int PAR, bool FULL>
__device__ __forceinline__ unsigned rho_sum_noted(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt,
                                                  int si, float4 ui, int q0, int q1, float &sum, float &comp) {
    const float rc2 = g.rc2_h;
    const f2 uixy = f2_pack(ui.x, ui.y);
    unsigned nb = 0;
#pragma unroll 2
    for (int j = 0; j < (FULL ? 32 : q1 - q0); j++) {
        const float4 D = nt.cand[PAR][q0 + j];
        const float4 uj = __ldg(s.u4 + si + __float_as_int(D.w));
        f2 dxy; float dz;
        const float r2 = pair_r2(uixy, ui.z, D, uj, dxy, dz);
        if (r2 < g.rcs2_h) {
            nb |= 1u << j;
            if (r2 < rc2) rho_pair(pt, r2, uj, sum, comp);
        }
    }
    return nb;
}
// the candidates q0 + j of the set bits j of `word` (a word of the group's list), in increasing order,
// so the in-range pairs are summed in the same order as by the full loop
template <int PAR>
__device__ __forceinline__ void rho_sum_listed(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt,
                                               int si, float4 ui, int q0, unsigned word, float &sum, float &comp) {
    const float rc2 = g.rc2_h;
    const f2 uixy = f2_pack(ui.x, ui.y);
    for (unsigned w = word; w; w &= w - 1) {
        const int j = __ffs(w) - 1;
        const float4 D = nt.cand[PAR][q0 + j];
        const float4 uj = __ldg(s.u4 + si + __float_as_int(D.w));
        f2 dxy; float dz;
        const float r2 = pair_r2(uixy, ui.z, D, uj, dxy, dz);
        if (r2 < rc2) rho_pair(pt, r2, uj, sum, comp);
    }
}
// Whether this density pass rebuilds the group lists: the same answer in every thread of the grid, as
// nothing it reads changes during the pass (all 32 lanes of the warp call it). The margin covers the
// FP32 rounding of the distances and of the sums, which is below 1e-5 half-lattice units.
constexpr float kSkinMargin = 1e-3f;
__device__ __forceinline__ bool skin_full(const Geom &g, const Slots &s) {
    if (!(g.skin_h > 0.f)) return true;
    const SkinState *k = s.skin;
    const int lane = threadIdx.x & 31;
    const unsigned m = __reduce_max_sync(0xffffffffu, max(k->step_max2[lane], k->step_max2[lane + 32]));
    const float step = sqrtf(__uint_as_float(m));
    return k->dirty != 0 || !(2.f * (k->acc + step) + kSkinMargin <= g.skin_h);
}
// the list of the 32-site group of parity par holding site u: kListWords words over the pruned candidates
__device__ __forceinline__ unsigned *group_list(const Geom &g, const Slots &s, int par, int u) {
    return s.near + kListWords * (par * ((g.n_local_half + 31) >> 5) + (u >> 5));
}

// lists: use the group lists (all 32 lanes of the warp call this, with valid false for threads past
// the end; the warp covers one 32-site group of one parity). full: visit every pruned candidate and
// rebuild the group's list; else visit the listed candidates only.
__device__ __forceinline__ void k_lat_rho_mixed_site(int t, bool valid, const NeighTables &nt, const Geom &g, const Slots &s, const Inter &in,
                                                     const PotTables &pt, bool hook, int order, bool lists, bool full) {
    int par = 0, u = 0;
    const int sl = valid ? gather_site(g, t, order, par, u) : -1;
    const int si = sl >= 0 ? sidx(g, sl) : 0;
    const float4 ui = sl >= 0 ? s.u4[si] : vacant_u4();
    const int ti = __float_as_int(ui.w);
    const unsigned live = lists ? __ballot_sync(0xffffffffu, ti >= 0) : 0u;
    // a site marked by a far or just recombined atom nearby makes its group rebuild its list: that
    // atom's record did not come from firststep, so the skin's bound does not cover it
    if (lists && !full) full = __any_sync(0xffffffffu, sl >= 0 && in.far_flag[sl]);
    if (sl < 0) return;
    if (ti < 0) { s.rho[sl] = 0.0; return; }
    float sum = 0.f, comp = 0.f;
    const int np = nt.npruned;
    if (lists) {  // 32 candidates per list word; the group's word: any live site of the warp
        unsigned *w = group_list(g, s, par, u);
        if (full) {
            const bool leader = (int) (threadIdx.x & 31) == __ffs(live) - 1;
            for (int k = 0; k * 32 < np; k++) {
                const int q0 = 32 * k, q1 = min(q0 + 32, np);
                const unsigned nb = q1 - q0 == 32 ? (par ? rho_sum_noted<1, true>(nt, g, s, pt, si, ui, q0, q1, sum, comp)
                                                         : rho_sum_noted<0, true>(nt, g, s, pt, si, ui, q0, q1, sum, comp))
                                                  : (par ? rho_sum_noted<1, false>(nt, g, s, pt, si, ui, q0, q1, sum, comp)
                                                         : rho_sum_noted<0, false>(nt, g, s, pt, si, ui, q0, q1, sum, comp));
                const unsigned any = __reduce_or_sync(live, nb);
                if (leader) w[k] = any;
            }
        } else {
            const uint4 n4 = *reinterpret_cast<const uint4 *>(w);
            for (int k = 0; k * 32 < np; k++) {
                const unsigned word = k == 0 ? n4.x : k == 1 ? n4.y : k == 2 ? n4.z : n4.w;
                if (par) rho_sum_listed<1>(nt, g, s, pt, si, ui, 32 * k, word, sum, comp);
                else rho_sum_listed<0>(nt, g, s, pt, si, ui, 32 * k, word, sum, comp);
            }
        }
    } else {
        if (par) rho_sum_mixed<1>(nt, g, s, pt, si, ui, 0, np, sum, comp);
        else rho_sum_mixed<0>(nt, g, s, pt, si, ui, 0, np, sum, comp);
    }
    if (in.far_flag[sl]) {
        const int nf = nt.nfull;
        if (par) rho_sum_mixed<1>(nt, g, s, pt, si, ui, np, nf, sum, comp);
        else rho_sum_mixed<0>(nt, g, s, pt, si, ui, np, nf, sum, comp);
    }
    const double rho = (double) sum - (double) comp;
    s.rho[sl] = rho;
    if (!hook && lattice_only(in)) {
        int m; float p;
        locate_f((float) rho, pt.inv_drho_f, pt.nrho, m, p);
        s.df32[si] = der_f(pt.F_dff + ti * pt.nrho, m, p);
    }
}
template <bool LOOP>  // LOOP: several sites per thread, one grid stride apart (no group lists)
__global__ void __launch_bounds__(512, 4) k_lat_rho_mixed(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, PotTables pt, bool hook, int order, int tbase,
                                                       int nthreads, bool lists) {
    const int t0 = tbase + blockIdx.x * blockDim.x + threadIdx.x;  // threads [tbase, nthreads)
    if (!LOOP) {
        const bool full = lists && skin_full(g, s);
        if (full && blockIdx.x == 0 && threadIdx.x == 0) s.skin->rebuilt = 1;
        k_lat_rho_mixed_site(t0, t0 < nthreads, nt, g, s, in, pt, hook, order, lists, full);
        return;
    }
    for (int t = t0; t < nthreads; t += gridDim.x * blockDim.x)
        k_lat_rho_mixed_site(t, true, nt, g, s, in, pt, hook, order, false, true);
}

// atoms per thread: each thread takes rho_apt sites, one grid stride apart (the stride is a multiple
// of 64, so warps keep their parity and thread order)
// The passes can keep and use per-group candidate lists when every warp of both passes covers one
// 32-site group of one parity: one site per thread, and (for the parity-major order) a multiple of 32
// sites per parity; the pruned candidates fit the list words.
bool lists_ok(const LaunchCtx &lc, const Geom &g) {
    const bool aligned = (g.n_local_half & 31) == 0;
    return lc.nt->npruned <= 32 * kListWords && lc.rho_apt == 1 && lc.force_apt == 1 && (lc.rho_order == 1 || aligned) &&
           (lc.force_order == 1 || aligned);
}
static void launch_lat_rho_threads(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, bool hook,
                                   int tb, int te, bool lists = false) {
    const int order = lc.rho_order, b = lc.rho_block;
    const int n = (te - tb + b * lc.rho_apt - 1) / (b * lc.rho_apt);
    if (n <= 0) return;
    if (lc.rho_apt > 1) {
        if (mixed) k_lat_rho_mixed<true><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, hook, order, tb, te, false);
        else k_lat_rho_fp64<true><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, hook, order, tb, te);
    } else {
        if (mixed) k_lat_rho_mixed<false><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, hook, order, tb, te, lists);
        else k_lat_rho_fp64<false><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, hook, order, tb, te);
    }
}
// one block of kSkinSlots threads
__global__ void __launch_bounds__(kSkinSlots) k_skin_advance(SkinState *k) {
    __shared__ unsigned wmax[kSkinSlots / 32];
    unsigned v = k->step_max2[threadIdx.x];
    k->step_max2[threadIdx.x] = 0u;
    v = __reduce_max_sync(0xffffffffu, v);
    if ((threadIdx.x & 31) == 0) wmax[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x != 0) return;
    unsigned m = 0u;
    for (int w = 0; w < kSkinSlots / 32; w++) m = max(m, wmax[w]);
    if (k->rebuilt) {  // built on this step's records: the sum restarts
        k->acc = 0.f;
        k->dirty = 0;
        k->rebuilt = 0;
        k->rebuilds++;
    } else {
        k->acc += sqrtf(__uint_as_float(m));  // a NaN or infinity forces the next pass to rebuild
    }
    k->passes++;
}
void launch_skin_advance(const LaunchCtx &lc, Slots s) { k_skin_advance<<<1, kSkinSlots, 0, lc.stream>>>(s.skin); }
void launch_skin_dirty(const LaunchCtx &lc, Slots s) { cudaMemsetAsync(&s.skin->dirty, 1, 1, lc.stream); }

// A mixed pass with the group lists is followed by the skin's advance. A mixed pass without them
// leaves the lists behind the positions, so the next pass with them rebuilds them.
void launch_lat_rho(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, bool hook, bool lists) {
    const bool v = lists && mixed && !hook && lists_ok(lc, g);
    launch_lat_rho_threads(lc, g, s, in, t, mixed, hook, 0, gather_threads(g, lc.rho_order), v);
    if (v) launch_skin_advance(lc, s);
    else if (mixed) launch_skin_dirty(lc, s);
}
// thread range of the sites [u0, u1) of both parities (u0, u1 multiples of 32, or u1 = n_local_half)
static void site_threads(const Geom &g, int order, int u0, int u1, int tb[2], int te[2], int &nr) {
    if (order) {  // warp w of parity p covers sites 32 (w / 2) .. + 31: thread t = 64 (u / 32) + 32 p + u % 32
        tb[0] = (u0 >> 5) << 6;
        te[0] = u1 >= g.n_local_half ? gather_threads(g, 1) : (u1 >> 5) << 6;
        nr = 1;
    } else {      // parity-major threads: one range per parity
        tb[0] = u0; te[0] = u1;
        tb[1] = g.n_local_half + u0; te[1] = g.n_local_half + u1;
        nr = 2;
    }
}
void launch_lat_rho_sites(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, int u0, int u1,
                          bool lists) {
    if (u1 <= u0) return;
    int tb[2], te[2], nr;
    site_threads(g, lc.rho_order, u0, u1, tb, te, nr);
    const bool v = lists && mixed && lists_ok(lc, g);
    for (int r = 0; r < nr; r++) launch_lat_rho_threads(lc, g, s, in, t, mixed, false, tb[r], te[r], v);
    if (!v && mixed) launch_skin_dirty(lc, s);  // the caller advances the skin after the last slab
}

// dF/drho when inter atoms added density after the lattice pass (or for the df hook)
template <bool MIXED>
__global__ void k_lat_df(Geom g, Slots s, Inter in, PotTables pt, bool hook) {
    if (!hook && lattice_only(in)) return;  // already fused into the density pass
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < g.n_local; t += gridDim.x * blockDim.x) {
        int i, j, k;
        const int sl = local_slot(g, t, i, j, k);
        const int ti = s.type[sl];
        if (ti < 0) continue;
        if (MIXED) {
            int m; float p;
            locate_f((float) s.rho[sl], pt.inv_drho_f, pt.nrho, m, p);
            s.df32[sidx(g, sl)] = der_f(pt.F_dff + ti * pt.nrho, m, p);
        } else {
            int m; double p;
            locate_d(s.rho[sl], pt.inv_drho, pt.nrho, m, p);
            s.df[sl] = der_d(pt.F_d + ti * pt.nrho, m, p);
        }
    }
}
void launch_lat_df(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, bool hook) {
    const int b = 256;
    const int n = hook ? (g.n_local + b - 1) / b : std::max(1, std::min(lc.num_sms * 8, (g.n_local + b - 1) / b));
    if (mixed) k_lat_df<true><<<n, b, 0, lc.stream>>>(g, s, in, t, hook);
    else k_lat_df<false><<<n, b, 0, lc.stream>>>(g, s, in, t, hook);
}

// ------------------------------------------------------------------------------------------------
// lattice force pass (atom::latForce, src/atom.cpp:311-358, as a full gather). When no inter atom
// adds force afterwards, the second half-kick (NewtonMotion::secondstep, src/newton_motion.cpp:57-67)
// is fused, and inside a fused graph (mixed form) so is the next loop body's firststep.
// fpair = -(F'_i rho'_j(r) + F'_j rho'_i(r) + phi'_ij(r)) / r, phi = (r phi) / r.
// ------------------------------------------------------------------------------------------------
template <int PAR>
__device__ __forceinline__ void force_sum_fp64(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt, int sl, int ti,
                                               int si, float4 ui, double xi, double yi, double zi, double dfi, int q0, int q1,
                                               double &fx, double &fy, double &fz) {
    const Knot64 *rho_di = pt.rho_d + ti * pt.nr;
    const f2 uixy = f2_pack(ui.x, ui.y);
#pragma unroll 2
    for (int q = q0; q < q1; q++) {
        const float4 D = nt.cand[PAR][q];
        const float4 uj = __ldg(s.u4 + si + __float_as_int(D.w));
        if (!near_f32(g, uixy, ui.z, D, uj)) continue;
        const int sj = sl + nt.lat[PAR][q];
        const int tj = __float_as_int(uj.w);
        const double dx = xi - s.x[sj], dy = yi - s.y[sj], dz = zi - s.z[sj];
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < g.rc2) {
            const double rinv = rsqrt(r2);
            const double r = r2 * rinv;
            int m; double p;
            locate_d(r, pt.inv_dr, pt.nr, m, p);
            const double rhojp = der_d(pt.rho_d + tj * pt.nr, m, p);
            const double rhoip = (tj == ti) ? rhojp : der_d(rho_di, m, p);
            const int pr = (ti * 3 + tj) * pt.nr;
            const double zv = val_d(pt.z_v + pr, m, p);
            const double zp = der_d(pt.z_d + pr, m, p);
            const double phi = zv * rinv;
            const double phip = zp * rinv - phi * rinv;
            const double psip = dfi * rhojp + s.df[sj] * rhoip + phip;
            const double fpair = -psip * rinv;
            fx += dx * fpair;
            fy += dy * fpair;
            fz += dz * fpair;
        }
    }
}

__device__ __forceinline__ void k_lat_force_fp64_site(int t, const NeighTables &nt, const Geom &g, const Slots &s, const Inter &in,
                                                const PotTables &pt, StepParams *sp, bool kick, bool hook, int order) {
    int par;
    const int sl = gather_slot(g, t, order, par);
    if (sl < 0) return;
    const int ti = s.type[sl];
    if (ti < 0) { s.fx[sl] = 0.0; s.fy[sl] = 0.0; s.fz[sl] = 0.0; return; }
    const double xi = s.x[sl], yi = s.y[sl], zi = s.z[sl];
    const double dfi = s.df[sl];
    const int si = sidx(g, sl);
    const float4 ui = s.u4[si];
    double fx = 0.0, fy = 0.0, fz = 0.0;
    const int np = nt.npruned;
    if (par) force_sum_fp64<1>(nt, g, s, pt, sl, ti, si, ui, xi, yi, zi, dfi, 0, np, fx, fy, fz);
    else force_sum_fp64<0>(nt, g, s, pt, sl, ti, si, ui, xi, yi, zi, dfi, 0, np, fx, fy, fz);
    if (in.far_flag[sl]) {
        const int nf = nt.nfull;
        if (par) force_sum_fp64<1>(nt, g, s, pt, sl, ti, si, ui, xi, yi, zi, dfi, np, nf, fx, fy, fz);
        else force_sum_fp64<0>(nt, g, s, pt, sl, ti, si, ui, xi, yi, zi, dfi, np, nf, fx, fy, fz);
    }
    s.fx[sl] = fx; s.fy[sl] = fy; s.fz[sl] = fz;
    if (kick && !hook && kick_in_lattice_pass(in, sl)) {
        const double c = dt_inv_m_of(sp, ti);
        const double vx = __dadd_rn(s.vx[sl], __dmul_rn(c, fx));
        const double vy = __dadd_rn(s.vy[sl], __dmul_rn(c, fy));
        const double vz = __dadd_rn(s.vz[sl], __dmul_rn(c, fz));
        s.vx[sl] = vx; s.vy[sl] = vy; s.vz[sl] = vz;
        if (variable_dt(sp)) note_vmax2(sp, speed2(vx, vy, vz));
    }
}
template <bool LOOP>  // LOOP: several sites per thread, one grid stride apart
__global__ void __launch_bounds__(512) k_lat_force_fp64(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, PotTables pt,
                                                         StepParams *sp, bool kick, bool hook, int order, int tbase,
                                                         int nthreads) {
    const int t0 = tbase + blockIdx.x * blockDim.x + threadIdx.x;  // threads [tbase, nthreads)
    if (!LOOP) {
        if (t0 < nthreads) k_lat_force_fp64_site(t0, nt, g, s, in, pt, sp, kick, hook, order);
        return;
    }
    for (int t = t0; t < nthreads; t += gridDim.x * blockDim.x) k_lat_force_fp64_site(t, nt, g, s, in, pt, sp, kick, hook, order);
}

// Compensated force sums of the mixed form: each pair term d * fpair is added by Kahan's method
// (W. Kahan, "Further remarks on reducing truncation errors", CACM 8(1), 1965). The running error is
// kept negated (m = -c), so the term's product and the correction fuse into one rounding
// (y = d * fpair + m) and a component costs four operations; x and y go through the packed f32x2
// forms. The sum's value is s + m.
struct ForceAcc {
    f2 sxy, mxy;  // running sums and their negated compensations, x and y packed
    float sz, mz;
};
__device__ __forceinline__ void force_acc_add(ForceAcc &a, f2 dxy, float dz, float fpair) {
    const f2 yxy = f2_fma(dxy, f2_pack(fpair, fpair), a.mxy);
    const f2 txy = f2_add(a.sxy, yxy);
    a.mxy = f2_sub(yxy, f2_sub(txy, a.sxy));
    a.sxy = txy;
    const float yz = __fmaf_rn(dz, fpair, a.mz);
    const float tz = __fadd_rn(a.sz, yz);
    a.mz = __fsub_rn(yz, __fsub_rn(tz, a.sz));
    a.sz = tz;
}

// one candidate of the force pass: the pair term when inside the cutoff (false for vacancies, NaN)
template <int PAR>
__device__ __forceinline__ void force_candidate(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt, int si,
                                                int ti, int fbase, f2 uixy, float uiz, float dfi, int q, ForceAcc &acc) {
    const float4 D = nt.cand[PAR][q];
    const int oj = si + __float_as_int(D.w);
    const float4 uj = __ldg(s.u4 + oj);
    f2 dxy; float dz;
    const float r2 = pair_r2(uixy, uiz, D, uj, dxy, dz);
    if (r2 < g.rc2_h) {
        const int tj = __float_as_int(uj.w);
        const float rinv_h = rsqrtf(r2);
        const float rp = r2 * rinv_h;
        int m; float p;
        locate_r_f(rp, pt.h_inv_dr_f, pt.nr, m, p);
        // record {c0, d0, c1, d1, c2, d2, c3, 0}: r*phi = c(p), rho_tj' = d(p), both in one Horner
        float z[8];
        ld_nc_v8(pt.zr8 + 8 * (fbase + tj * pt.nr + m), z);
        const f2 pp = f2_pack(p, p);
        f2 h = f2_fma(f2_pack(z[6], z[7]), pp, f2_pack(z[4], z[5]));
        h = f2_fma(h, pp, f2_pack(z[2], z[3]));
        h = f2_fma(h, pp, f2_pack(z[0], z[1]));
        float zv, rhojp;
        f2_unpack(h, zv, rhojp);
        const float zp = fmaf(fmaf(3.0f * z[6], p, z[4] + z[4]), p, z[2]) * pt.inv_dr_f;
        const float rhoip = (tj == ti) ? rhojp : der_f(pt.rho_dff + ti * pt.nr, m, p);
        const float rinv = rinv_h * g.inv_h_f;
        const float phi = zv * rinv;
        const float phip = (zp - phi) * rinv;
        const float psip = dfi * rhojp + __ldg(s.df32 + oj) * rhoip + phip;
        const float fpair = -psip * rinv;
        force_acc_add(acc, dxy, dz, fpair);
    }
}
template <int PAR>
__device__ __forceinline__ void force_sum_mixed(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt, int si, int ti,
                                                float4 ui, float dfi, int q0, int q1, ForceAcc &acc) {
    // records of the pair row ti; the table constants are read from the parameter bank where used
    const int fbase = (ti * 3) * pt.nr;
    const f2 uixy = f2_pack(ui.x, ui.y);
#pragma unroll 1  // 2, 3, 4 and full unrolling measured slower
    for (int q = q0; q < q1; q++) force_candidate<PAR>(nt, g, s, pt, si, ti, fbase, uixy, ui.z, dfi, q, acc);
}
// the candidates of the warp's group list, in table order: the density pass of this step checked or
// rebuilt the list, so it holds every pruned candidate inside the cutoff for any site of the group
// (the cutoff is tested again here with the same rounding, so the pairs summed are those of the full
// loop, in the same order)
template <int PAR>
__device__ __forceinline__ void force_sum_listed(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt, int si,
                                                 int ti, float4 ui, float dfi, const unsigned *words, ForceAcc &acc) {
    const int fbase = (ti * 3) * pt.nr;
    const f2 uixy = f2_pack(ui.x, ui.y);
    for (int k = 0; k * 32 < nt.npruned; k++)
        for (unsigned w = words[k]; w; w &= w - 1)
            force_candidate<PAR>(nt, g, s, pt, si, ti, fbase, uixy, ui.z, dfi, 32 * k + __ffs(w) - 1, acc);
}

// local coordinates and local index (k, j, i order) of a local slot
__device__ __forceinline__ int local_index_of(const Geom &g, int sl, int &i, int &j, int &k) {
    const int X = sl % g.Sx, r = sl / g.Sx;
    i = X - g.gx;
    j = r % g.Sy - g.gy;
    k = r / g.Sy - g.gz;
    return (k * g.by + j) * g.bx + i;
}

__device__ __forceinline__ void k_lat_force_mixed_site(int t, const NeighTables &nt, const Geom &g, const Slots &s, const Inter &in,
                                                const PotTables &pt, StepParams *sp, bool kick, bool hook, int order,
                                                bool fuse_next, bool lists) {
    int par, u;
    const int sl = gather_site(g, t, order, par, u);
    if (sl < 0) return;
    const int si = sidx(g, sl);
    const float4 ui = s.u4[si];
    const int ti = __float_as_int(ui.w);
    if (ti < 0) {
        s.fx[sl] = 0.0; s.fy[sl] = 0.0; s.fz[sl] = 0.0;
        if (fuse_next && lattice_only(in)) {  // the next firststep's flag and record of a vacancy
            int i, j, k;
            in.dflag[local_index_of(g, sl, i, j, k)] = 0;
            s.u4n[si] = vacant_u4();
        }
        return;
    }
    const float dfi = s.df32[si];
    // compensated force sums (x and y packed, z)
    ForceAcc acc{f2_pack(0.f, 0.f), f2_pack(0.f, 0.f), 0.f, 0.f};
    const int np = nt.npruned;
    if (lists) {
        const unsigned *w = group_list(g, s, par, u);
        if (par) force_sum_listed<1>(nt, g, s, pt, si, ti, ui, dfi, w, acc);
        else force_sum_listed<0>(nt, g, s, pt, si, ti, ui, dfi, w, acc);
    } else {
        if (par) force_sum_mixed<1>(nt, g, s, pt, si, ti, ui, dfi, 0, np, acc);
        else force_sum_mixed<0>(nt, g, s, pt, si, ti, ui, dfi, 0, np, acc);
    }
    if (in.far_flag[sl]) {
        const int nf = nt.nfull;
        if (par) force_sum_mixed<1>(nt, g, s, pt, si, ti, ui, dfi, np, nf, acc);
        else force_sum_mixed<0>(nt, g, s, pt, si, ti, ui, dfi, np, nf, acc);
    }
    // each sum with its compensation, converted to FP64 once
    float sx, sy, mx, my;
    f2_unpack(acc.sxy, sx, sy);
    f2_unpack(acc.mxy, mx, my);
    const double h = 0.5 * g.a0;
    const double fx = h * ((double) sx + (double) mx);
    const double fy = h * ((double) sy + (double) my);
    const double fz = h * ((double) acc.sz + (double) acc.mz);
    const bool fused = fuse_next && kick && !hook && lattice_only(in);
    // a fused body's forces are used only in registers: the next body's firststep is taken here, and
    // the last body of a graph (never fused) stores the forces the state keeps between launches
    if (!fused) { s.fx[sl] = fx; s.fy[sl] = fy; s.fz[sl] = fz; }
    if (kick && !hook && kick_in_lattice_pass(in, sl)) {
        const double c = dt_inv_m_of(sp, ti);
        const double vx = __dadd_rn(s.vx[sl], __dmul_rn(c, fx));
        const double vy = __dadd_rn(s.vy[sl], __dmul_rn(c, fy));
        const double vz = __dadd_rn(s.vz[sl], __dmul_rn(c, fz));
        if (!fused) { s.vx[sl] = vx; s.vy[sl] = vy; s.vz[sl] = vz; }  // else first_half writes the next v
        if (variable_dt(sp)) note_vmax2(sp, speed2(vx, vy, vz));
        if (fused) {
            // the next loop body's firststep for this atom, with the force still in registers (the
            // other threads of this pass still read this atom's u4, so the new record goes to the next
            // body's buffer, u4n)
            int i, j, k;
            const int tl = local_index_of(g, sl, i, j, k);
            first_half<true, true>(g, s, in, sp, sl, tl, i, j, k, ti, vx, vy, vz, fx, fy, fz, s.u4n, s.u4);
        }
    }
}
template <bool LOOP>  // LOOP: several sites per thread, one grid stride apart
__global__ void __launch_bounds__(512, 3) k_lat_force_mixed(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, PotTables pt,
                                                         StepParams *sp, bool kick, bool hook, int order, int tbase,
                                                         int nthreads, bool fuse_next, bool lists) {
    const int t0 = tbase + blockIdx.x * blockDim.x + threadIdx.x;  // threads [tbase, nthreads)
    if (!LOOP) {
        if (t0 < nthreads) k_lat_force_mixed_site(t0, nt, g, s, in, pt, sp, kick, hook, order, fuse_next, lists);
        return;
    }
    for (int t = t0; t < nthreads; t += gridDim.x * blockDim.x)
        k_lat_force_mixed_site(t, nt, g, s, in, pt, sp, kick, hook, order, fuse_next, false);
}

static void launch_lat_force_threads(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, StepParams *p,
                                     bool kick, bool mixed, bool hook, int tb, int te, bool fuse_next = false,
                                     bool lists = false) {
    const int order = lc.force_order, b = lc.force_block;
    const int n = (te - tb + b * lc.force_apt - 1) / (b * lc.force_apt);
    if (n <= 0) return;
    const bool fuse = fuse_next && mixed && kick && !hook;
    if (lc.force_apt > 1) {
        if (mixed) k_lat_force_mixed<true><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, p, kick, hook, order, tb, te, fuse, false);
        else k_lat_force_fp64<true><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, p, kick, hook, order, tb, te);
    } else {
        if (mixed) k_lat_force_mixed<false><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, p, kick, hook, order, tb, te, fuse, lists);
        else k_lat_force_fp64<false><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, p, kick, hook, order, tb, te);
    }
}
void launch_lat_force(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, StepParams *p, bool kick,
                      bool mixed, bool hook, bool fuse_next, bool lists) {
    launch_lat_force_threads(lc, g, s, in, t, p, kick, mixed, hook, 0, gather_threads(g, lc.force_order), fuse_next,
                             lists && mixed && !hook && lists_ok(lc, g));
}
void launch_lat_force_sites(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, StepParams *p, bool kick,
                            bool mixed, int u0, int u1, bool lists) {
    if (u1 <= u0) return;
    int tb[2], te[2], nr;
    site_threads(g, lc.force_order, u0, u1, tb, te, nr);
    const bool v = lists && mixed && lists_ok(lc, g);
    for (int r = 0; r < nr; r++) launch_lat_force_threads(lc, g, s, in, t, p, kick, mixed, false, tb[r], te[r], false, v);
}

// second half-kick for lattice slots (only when inter atoms prevented fusion, or always) and for
// inter atoms (src/newton_motion.cpp:57-74)
__global__ void k_secondstep(Geom g, Slots s, Inter in, StepParams *p, int lattice_mode) {
    const int n_inter = in.cnt[CNT_INTER];
    // mode 2 (after a kicking force pass): the lattice atoms were kicked by the lattice force pass or,
    // for the owners of inter-atom pairs, by the owner gather; inter atoms only
    const bool lattice = lattice_mode == 1;
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    double v2max = 0.0;
    if (lattice) {
        for (int t = t0; t < g.n_local; t += stride) {
            int i, j, k;
            const int sl = local_slot(g, t, i, j, k);
            const int ty = s.type[sl];
            if (ty < 0) continue;
            const double c = dt_inv_m_of(p, ty);
            const double vx = __dadd_rn(s.vx[sl], __dmul_rn(c, s.fx[sl]));
            const double vy = __dadd_rn(s.vy[sl], __dmul_rn(c, s.fy[sl]));
            const double vz = __dadd_rn(s.vz[sl], __dmul_rn(c, s.fz[sl]));
            s.vx[sl] = vx; s.vy[sl] = vy; s.vz[sl] = vz;
            v2max = fmax(v2max, speed2(vx, vy, vz));
        }
    }
    for (int a = t0; a < n_inter; a += stride) {
        const double c = dt_inv_m_of(p, in.type[a]);
        const double vx = __dadd_rn(in.vx[a], __dmul_rn(c, in.fx[a]));
        const double vy = __dadd_rn(in.vy[a], __dmul_rn(c, in.fy[a]));
        const double vz = __dadd_rn(in.vz[a], __dmul_rn(c, in.fz[a]));
        in.vx[a] = vx; in.vy[a] = vy; in.vz[a] = vz;
        v2max = fmax(v2max, speed2(vx, vy, vz));
    }
    if (v2max > 0.0) note_vmax2(p, v2max);
}
// grid-stride kernels that often have nothing to do: a grid no larger than the box needs, so a
// small box does not schedule a thousand idle blocks every step
inline int box_grid(const LaunchCtx &lc, const Geom &g, int per_sm, int threads) {
    return std::max(1, std::min(lc.num_sms * per_sm, (g.n_local + threads - 1) / threads));
}
void launch_secondstep(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, StepParams *p, bool lattice) {
    k_secondstep<<<box_grid(lc, g, 8, 256), 256, 0, lc.stream>>>(g, s, in, p, lattice ? 1 : 2);
}

// ------------------------------------------------------------------------------------------------
// timestep control (extension: the reference sets dt per stage, src/newton_motion.cpp:13-28)
// ------------------------------------------------------------------------------------------------
// dt/(2m) per type as NewtonMotion::preComputeDtInv2m computes it: (0.5 * dt * ftm2v) / m
__device__ __forceinline__ void set_dt_dev(StepParams *p, double dt) {
    p->dt = dt;
    const double dt_halve = __dmul_rn(__dmul_rn(0.5, dt), kFtm2v);
    for (int t = 0; t < 3; t++) p->dt_inv_m[t] = __ddiv_rn(dt_halve, c_mass[t]);
}
__global__ void k_set_step(StepParams *p, double dt, double dx_max, double dt_min, double dt_max) {
    p->dx_max = dx_max;
    p->dt_min = dt_min;
    p->dt_max = dt_max;
    set_dt_dev(p, dt);
}
void launch_set_step(const LaunchCtx &lc, StepParams *sp, double dt, double dx_max, double dt_min, double dt_max) {
    k_set_step<<<1, 1, 0, lc.stream>>>(sp, dt, dx_max, dt_min, dt_max);
}
// One block of kVmaxSlots threads: reduce and clear the max words, then (variable mode)
// dt = clamp(dx_max / sqrt(max |v|^2), dt_min, dt_max); record dt and advance the clock.
__global__ void __launch_bounds__(kVmaxSlots) k_step_head(StepParams *p) {
    __shared__ unsigned long long part[kVmaxSlots / 32];
    const unsigned long long b = p->vmax2[threadIdx.x];
    p->vmax2[threadIdx.x] = 0ull;
    const unsigned hi = (unsigned) (b >> 32), lo = (unsigned) b;
    const unsigned mhi = __reduce_max_sync(0xffffffffu, hi);
    const unsigned mlo = __reduce_max_sync(0xffffffffu, hi == mhi ? lo : 0u);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = ((unsigned long long) mhi << 32) | mlo;
    __syncthreads();
    if (threadIdx.x != 0) return;
    unsigned long long m = 0ull;
    for (int w = 0; w < kVmaxSlots / 32; w++) m = part[w] > m ? part[w] : m;
    if (p->dx_max > 0.0) {
        const double v2 = __longlong_as_double((long long) m);
        double dt = v2 > 0.0 ? __ddiv_rn(p->dx_max, __dsqrt_rn(v2)) : p->dt_max;
        if (dt < p->dt_min) dt = p->dt_min;
        if (dt > p->dt_max) dt = p->dt_max;
        set_dt_dev(p, dt);
    }
    const long long k = p->steps;
    p->hist[k % kDtHistory] = p->dt;
    p->time = __dadd_rn(p->time, p->dt);
    p->steps = k + 1;
}
void launch_step_head(const LaunchCtx &lc, StepParams *sp) { k_step_head<<<1, kVmaxSlots, 0, lc.stream>>>(sp); }
// steps taken and simulated time into a sample record (stage machine thermo output)
__global__ void k_clock_sample(const StepParams *p, double *out) {
    out[0] = (double) p->steps;
    out[1] = p->time;
}
void launch_clock_sample(const LaunchCtx &lc, const StepParams *sp, double *out) {
    k_clock_sample<<<1, 1, 0, lc.stream>>>(sp, out);
}
// max |v|^2 over local lattice atoms and local inter atoms, from scratch
__global__ void k_vmax_full(Geom g, Slots s, Inter in, StepParams *p) {
    const int stride = gridDim.x * blockDim.x;
    const int t0 = blockIdx.x * blockDim.x + threadIdx.x;
    double v2max = 0.0;
    for (int t = t0; t < g.n_local; t += stride) {
        int i, j, k;
        const int sl = local_slot(g, t, i, j, k);
        if (s.type[sl] < 0) continue;
        v2max = fmax(v2max, speed2(s.vx[sl], s.vy[sl], s.vz[sl]));
    }
    const int n_inter = in.cnt[CNT_INTER];
    for (int a = t0; a < n_inter; a += stride) v2max = fmax(v2max, speed2(in.vx[a], in.vy[a], in.vz[a]));
    if (v2max > 0.0) note_vmax2(p, v2max);
}
void launch_vmax_full(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, StepParams *sp) {
    cudaMemsetAsync(reinterpret_cast<char *>(sp) + offsetof(StepParams, vmax2), 0, sizeof(unsigned long long) * kVmaxSlots,
                    lc.stream);
    k_vmax_full<<<lc.num_sms * 8, 256, 0, lc.stream>>>(g, s, in, sp);
}

// ------------------------------------------------------------------------------------------------
// per-atom energy (extension): e_i = F(rho_i) + 1/2 sum_j phi_ij over lattice neighbours
// ------------------------------------------------------------------------------------------------
template <int PAR>
__device__ __forceinline__ double energy_sum_fp64(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt, int sl, int ti,
                                                  int q0, int q1) {
    const double xi = s.x[sl], yi = s.y[sl], zi = s.z[sl];
    double acc = 0.0;
    for (int q = q0; q < q1; q++) {
        const int sj = sl + nt.lat[PAR][q];
        const int tj = s.type[sj];
        if (tj < 0) continue;
        const double dx = xi - s.x[sj], dy = yi - s.y[sj], dz = zi - s.z[sj];
        const double r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < g.rc2) {
            const double rinv = rsqrt(r2);
            int m; double p;
            locate_d(r2 * rinv, pt.inv_dr, pt.nr, m, p);
            acc += val_d(pt.z_v + (ti * 3 + tj) * pt.nr, m, p) * rinv;
        }
    }
    return acc;
}
template <int PAR>
__device__ __forceinline__ void energy_sum_mixed(const NeighTables &nt, const Geom &g, const Slots &s, const PotTables &pt, int si, int ti,
                                                 float4 ui, int q0, int q1, float &sum, float &comp) {
    const float inv_h = 1.0f / g.h_f;
    for (int q = q0; q < q1; q++) {
        const float4 D = nt.cand[PAR][q];
        const float4 uj = __ldg(s.u4 + si + __float_as_int(D.w));
        const float dx = (ui.x - uj.x) - D.x, dy = (ui.y - uj.y) - D.y, dz = (ui.z - uj.z) - D.z;
        const float r2 = dx * dx + dy * dy + dz * dz;
        if (r2 < g.rc2_h) {  // false for vacancies (NaN coordinates)
            const int tj = __float_as_int(uj.w);
            const float rinv_h = rsqrtf(r2);
            int m; float p;
            locate_f(r2 * rinv_h, pt.h_inv_dr_f, pt.nr, m, p);
            kahan(sum, comp, val_f(pt.z_vf + (ti * 3 + tj) * pt.nr, m, p) * (rinv_h * inv_h));
        }
    }
}

template <bool MIXED>
__global__ void __launch_bounds__(256) k_energy(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, PotTables pt, int order) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int par;
    const int sl = gather_slot(g, t, order, par);
    if (sl < 0) return;
    const int ti = s.type[sl];
    if (ti < 0) { s.e[sl] = 0.0; return; }
    const int np = nt.npruned;
    const int nq = in.far_flag[sl] ? nt.nfull : np;
    if (!MIXED) {
        double acc = par ? energy_sum_fp64<1>(nt, g, s, pt, sl, ti, 0, np) : energy_sum_fp64<0>(nt, g, s, pt, sl, ti, 0, np);
        if (nq > np) acc += par ? energy_sum_fp64<1>(nt, g, s, pt, sl, ti, np, nq) : energy_sum_fp64<0>(nt, g, s, pt, sl, ti, np, nq);
        int m; double p;
        locate_d(s.rho[sl], pt.inv_drho, pt.nrho, m, p);
        s.e[sl] = val_d(pt.F_v + ti * pt.nrho, m, p) + 0.5 * acc;
    } else {
        const int si = sidx(g, sl);
        const float4 ui = s.u4[si];
        float sum = 0.f, comp = 0.f;
        if (par) energy_sum_mixed<1>(nt, g, s, pt, si, ti, ui, 0, np, sum, comp);
        else energy_sum_mixed<0>(nt, g, s, pt, si, ti, ui, 0, np, sum, comp);
        if (nq > np) {
            if (par) energy_sum_mixed<1>(nt, g, s, pt, si, ti, ui, np, nq, sum, comp);
            else energy_sum_mixed<0>(nt, g, s, pt, si, ti, ui, np, nq, sum, comp);
        }
        int m; float p;
        locate_f((float) s.rho[sl], pt.inv_drho_f, pt.nrho, m, p);
        s.e[sl] = (double) val_f(pt.F_vf + ti * pt.nrho, m, p) + 0.5 * ((double) sum - (double) comp);
    }
}
void launch_energy(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed) {
    const int b = 256, n = (gather_threads(g, 0) + b - 1) / b;
    if (mixed) k_energy<true><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, 0);
    else k_energy<false><<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t, 0);
}

// ------------------------------------------------------------------------------------------------
// Far atoms: lattice atoms farther than 0.2 a0 from their site (after decide, only recombined
// atoms). Pairs beyond the pruned table can reach them, so the atom itself and the owner of every
// slot of its full neighbourhood get far_flag = 1: their gathers also run the tail of the table.
// (A normal atom k sees a far atom i across the periodic boundary through i's ghost image; k is the
// owner of a ghost slot in i's neighbourhood, so it is marked too.) Clearing writes 0 over the same
// slots of the old list. Work item e of a flat loop covers (far atom e / (nfull + 1), entry).
// ------------------------------------------------------------------------------------------------
__device__ void mark_far_neighbourhoods(const NeighTables &nt, const Geom &g, const Inter &in, int a0, int a1, int8_t v, int t0,
                                        int stride) {
    const int per = nt.nfull + 1;
    const int total = (a1 - a0) * per;
    for (int e = t0; e < total; e += stride) {
        const int sl = in.far_list[a0 + e / per];
        const int q = e % per;
        const int par = (sl % g.Sx) & 1;
        const int sj = q == nt.nfull ? sl : sl + (par ? nt.lat[1][q] : nt.lat[0][q]);
        in.far_flag[owner_slot(g, sj)] = v;
    }
}

// ------------------------------------------------------------------------------------------------
// Inter-atom list management: one block, so the reference's list order is kept exactly.
//   decide (src/atom.cpp:21-84), exchangeInter (src/pack/inter_particle_packer.cpp),
//   borderInter (src/pack/inter_border_packer.cpp), makeIndex (src/atom/inter_atom_list.cpp:27-45).
// ------------------------------------------------------------------------------------------------
constexpr int kManageThreads = 1024;

// exclusive block scan of one int per thread; returns the block total
__device__ int block_exclusive_scan(int v, int &excl) {
    __shared__ int warp_tot[32];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    int x = v;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[w] = x;
    __syncthreads();
    if (w == 0) {
        int t = (lane < (int) (blockDim.x >> 5)) ? warp_tot[lane] : 0;
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        warp_tot[lane] = t;  // inclusive
    }
    __syncthreads();
    const int warp_excl = w > 0 ? warp_tot[w - 1] : 0;
    excl = warp_excl + x - v;
    const int total = warp_tot[(blockDim.x >> 5) - 1];
    __syncthreads();
    return total;
}

// bitonic sort of n 64-bit keys in global memory by one block; buf capacity >= next pow2(n)
__device__ void block_bitonic_sort(long long *buf, int n) {
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = n + threadIdx.x; i < P; i += blockDim.x) buf[i] = LLONG_MAX;
    __syncthreads();
    for (int kk = 2; kk <= P; kk <<= 1) {
        for (int jj = kk >> 1; jj > 0; jj >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ jj;
                if (l > i) {
                    const long long a = buf[i], b = buf[l];
                    const bool up = (i & kk) == 0;
                    if ((a > b) == up) { buf[i] = b; buf[l] = a; }
                }
            }
            __syncthreads();
        }
    }
}

// the same sort in shared memory (sm holds at least next_pow2(n) keys)
__device__ void block_bitonic_sort_smem(long long *buf, int n, long long *sm) {
    int P = 1;
    while (P < n) P <<= 1;
    for (int i = threadIdx.x; i < P; i += blockDim.x) sm[i] = i < n ? buf[i] : LLONG_MAX;
    __syncthreads();
    for (int kk = 2; kk <= P; kk <<= 1) {
        for (int jj = kk >> 1; jj > 0; jj >>= 1) {
            for (int i = threadIdx.x; i < P; i += blockDim.x) {
                const int l = i ^ jj;
                if (l > i) {
                    const long long a = sm[i], b = sm[l];
                    const bool up = (i & kk) == 0;
                    if ((a > b) == up) { sm[i] = b; sm[l] = a; }
                }
            }
            __syncthreads();
        }
    }
    for (int i = threadIdx.x; i < n; i += blockDim.x) buf[i] = sm[i];
    __syncthreads();
}

// inter record move helpers (scratch layout: 13 doubles per record)
__device__ __forceinline__ void inter_save(const Inter &in, int a, int dst) {
    double *d = in.scratch_d + 13 * dst;
    d[0] = in.x[a]; d[1] = in.y[a]; d[2] = in.z[a];
    d[3] = in.vx[a]; d[4] = in.vy[a]; d[5] = in.vz[a];
    d[6] = in.fx[a]; d[7] = in.fy[a]; d[8] = in.fz[a];
    d[9] = in.rho[a]; d[10] = in.df[a]; d[11] = 0.0; d[12] = 0.0;
    in.scratch_u[dst] = in.id[a];
    in.scratch_i[dst] = in.type[a];
}
__device__ __forceinline__ void inter_restore(const Inter &in, int src, int a) {
    const double *d = in.scratch_d + 13 * src;
    in.x[a] = d[0]; in.y[a] = d[1]; in.z[a] = d[2];
    in.vx[a] = d[3]; in.vy[a] = d[4]; in.vz[a] = d[5];
    in.fx[a] = d[6]; in.fy[a] = d[7]; in.fz[a] = d[8];
    in.rho[a] = d[9]; in.df[a] = d[10];
    in.id[a] = in.scratch_u[src];
    in.type[a] = in.scratch_i[src];
}

__device__ __forceinline__ void region_fw(const Geom &g, int d, int dir, int lo[3], int hi[3]) {
    const int gg[3] = {g.gx, g.gy, g.gz}, bb[3] = {g.bx, g.by, g.bz}, ee[3] = {g.Sx, g.Sy, g.Sz};
    for (int q = 0; q < 3; q++) { lo[q] = 0; hi[q] = ee[q]; }
    for (int q = d + 1; q < 3; q++) { lo[q] = gg[q]; hi[q] = gg[q] + bb[q]; }
    if (dir == 0) { lo[d] = gg[d]; hi[d] = 2 * gg[d]; }
    else { lo[d] = bb[d]; hi[d] = bb[d] + gg[d]; }
}

// borderInter's entries: the local inter atoms, then the ghost images made so far
__device__ __forceinline__ void border_entry(const Inter &in, int n_loc, int e, double p3[3], int &ty, int &root) {
    if (e < n_loc) {
        p3[0] = in.x[e]; p3[1] = in.y[e]; p3[2] = in.z[e];
        ty = in.type[e];
        root = e;
    } else {
        const int k = e - n_loc;
        p3[0] = in.gx[k]; p3[1] = in.gy[k]; p3[2] = in.gz[k];
        ty = in.gtype[k];
        root = in.groot[k];
    }
}
// bit r set: the entry's nearest site lies in the region sent to direction r
__device__ __forceinline__ int border_regions(const Geom &g, const int lo[2][3], const int hi[2][3], const double p3[3]) {
    long long c[3];
    near_lat_coord(g, p3[0], p3[1], p3[2], c);
    int m = 0;
    for (int r = 0; r < 2; r++)
        if (c[0] >= lo[r][0] && c[0] < hi[r][0] && c[1] >= lo[r][1] && c[1] < hi[r][1] && c[2] >= lo[r][2] &&
            c[2] < hi[r][2])
            m |= 1 << r;
    return m;
}
// ghost image q of an entry, shifted by sh along d (past the capacity: the overflow error)
__device__ __forceinline__ void border_put(Inter &in, int q, const double p3[3], int d, double sh, int ty, int root) {
    if (q >= in.gcap) {
        set_error(in, MG_DEVERR_GHOST_OVERFLOW);
        return;
    }
    double p[3] = {p3[0], p3[1], p3[2]};
    p[d] = __dadd_rn(p[d], sh);
    in.gx[q] = p[0]; in.gy[q] = p[1]; in.gz[q] = p[2];
    in.gtype[q] = ty;
    in.groot[q] = root;
    in.gdf[q] = 0.0;
}

__global__ void __launch_bounds__(kManageThreads) k_inter_manage(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, int mask, bool mixed) {
    const int tid = threadIdx.x, nthr = blockDim.x;

    // The list counts are read once, by all threads before any is written, and then followed in
    // registers: every change to them is block-uniform (scan totals), and one global round trip
    // costs this single block about a microsecond. Thread 0 writes each change back for the
    // kernels that follow.
    int n_inter = in.cnt[CNT_INTER], n_ghost = in.cnt[CNT_GHOST];
    const int n_disp = in.cnt[CNT_DISPLACED];
    // The usual step of a crystal: no inter atom, no ghost image and nothing displaced, so every
    // phase would find its lists empty; what remains is decide voiding the previous step's far list
    // and the index being empty.
    const bool idle = n_inter == 0 && n_ghost == 0 && n_disp == 0;
    __syncthreads();
    if (idle) {
        if (tid == 0) {
            if (mask & MANAGE_DECIDE) in.cnt[CNT_FAR] = 0;
            if (mask & MANAGE_INDEX) *in.n_bucket = 0;
        }
        return;
    }

    if (mask & MANAGE_CLEAR_GHOST) {
        n_ghost = 0;
        if (tid == 0) in.cnt[CNT_GHOST] = 0;
    }

    if (mask & MANAGE_DECIDE) {
        // the far list of the previous step is void (its marks were cleared before this kernel)
        if (tid == 0) in.cnt[CNT_FAR] = 0;
        __syncthreads();
        // (i) displaced lattice atoms join the list in scan order (the collected list is ordered)
        int nd = n_disp;
        if (nd > in.dcap) nd = in.dcap;
        const int n0 = n_inter;
        if (nd > 0) {
            int room = in.cap - n0;
            if (nd > room) { if (tid == 0) set_error(in, MG_DEVERR_INTER_OVERFLOW); nd = room; }
            for (int q = tid; q < nd; q += nthr) {
                const int sl = in.displaced[q];
                const int a = n0 + q;
                in.id[a] = s.id[sl];
                in.type[a] = s.type[sl];
                in.x[a] = s.x[sl]; in.y[a] = s.y[sl]; in.z[a] = s.z[sl];
                in.vx[a] = s.vx[sl]; in.vy[a] = s.vy[sl]; in.vz[a] = s.vz[sl];
                in.fx[a] = s.fx[sl]; in.fy[a] = s.fy[sl]; in.fz[a] = s.fz[sl];
                in.rho[a] = s.rho[sl];
                in.df[a] = mixed ? (double) s.df32[sidx(g, sl)] : s.df[sl];
                s.type[sl] = kInvalid;
                s.vx[sl] = 0.0; s.vy[sl] = 0.0; s.vz[sl] = 0.0;
                s.u4[sidx(g, sl)] = vacant_u4();
            }
            __syncthreads();
            n_inter = n0 + nd;
            if (tid == 0) in.cnt[CNT_INTER] = n_inter;
        }
        if (tid == 0) in.cnt[CNT_DISPLACED] = 0;
        __syncthreads();

        // (ii) recombination with vacancies, first claimant in list order wins
        const int n = n_inter;
        int *cand = in.scratch_i + in.cap;  // n ints
        for (int a = tid; a < n; a += nthr) {
            const int near = near_index_in_sub_box(g, in.x[a], in.y[a], in.z[a]);
            int c = -1;
            if (near >= 0 && s.type[near] == kInvalid && is_out_box(g, s.x[near], s.y[near], s.z[near]) == kInBox) {
                c = near;
                atomicMin(&in.claim[near], a);
            }
            cand[a] = c;
        }
        __syncthreads();
        int *won = in.scratch_i + in.cap + in.cap;  // n ints
        int any_won = 0;
        for (int a = tid; a < n; a += nthr) {
            won[a] = (cand[a] >= 0 && in.claim[cand[a]] == a) ? 1 : 0;
            any_won |= won[a];
        }
        const bool recombined = __syncthreads_or(any_won);
        for (int a = tid; a < n; a += nthr) if (cand[a] >= 0) in.claim[cand[a]] = INT_MAX;
        // nobody recombined (the usual step): the compaction would rewrite the list unchanged
        if (recombined) {
            for (int a = tid; a < n; a += nthr) {
                if (!won[a]) continue;
                const int sl = cand[a];
                s.id[sl] = in.id[a];
                s.type[sl] = (int8_t) in.type[a];
                s.x[sl] = in.x[a]; s.y[sl] = in.y[a]; s.z[sl] = in.z[a];
                s.vx[sl] = in.vx[a]; s.vy[sl] = in.vy[a]; s.vz[sl] = in.vz[a];
                {
                    const int X = sl % g.Sx, r = sl / g.Sx, Y = r % g.Sy, Z = r / g.Sy;
                    double xs, ys, zs;
                    site_of(g, X, Y, Z, xs, ys, zs);
                    s.u4[sidx(g, sl)] = make_u4(g, in.x[a], in.y[a], in.z[a], xs, ys, zs, in.type[a]);
                }
                // A recombined atom may sit up to sqrt(5)/4 a0 from its new site. Every recombined atom
                // joins this step's far list: the marks on its neighbourhood also make the density pass
                // rebuild the candidate lists of the groups that can see it (its record did not come
                // from firststep). The tail pairs the marks add for an atom within 0.2 a0 of its site
                // are all beyond the cutoff, so they change no sum.
                {
                    const int q = atomicAdd(&in.cnt[CNT_FAR], 1);
                    if (q < in.fcap) in.far_list[q] = sl;
                    else set_error(in, MG_DEVERR_DISPLACED_OVERFLOW);
                }
            }
            __syncthreads();
            // stable compaction of the survivors
            int base = 0;
            for (int c0 = 0; c0 < n; c0 += nthr) {
                const int a = c0 + tid;
                const int keep = (a < n && !won[a]) ? 1 : 0;
                int ex;
                const int tot = block_exclusive_scan(keep, ex);
                if (keep) inter_save(in, a, base + ex);
                base += tot;
            }
            __syncthreads();
            for (int a = tid; a < base; a += nthr) inter_restore(in, a, a);
            n_inter = base;
            if (tid == 0) in.cnt[CNT_INTER] = base;
        }
        __syncthreads();
    }

    if (mask & MANAGE_EXCHANGE) {
        const uint32_t lowf[3] = {kXLow, kYLow, kZLow}, highf[3] = {kXHigh, kYHigh, kZHigh};
        // an atom's out-of-box flags are found once and kept until a partition moves and shifts the
        // records (each thread keeps the same atoms from one dimension to the next)
        uint32_t *flags = reinterpret_cast<uint32_t *>(in.scratch_i + 2 * in.cap);
        bool flags_valid = false;
        for (int d = 0; d < 3; d++) {
            const int n = n_inter;
            int *cls = in.scratch_i + in.cap;  // 0 stay, 1 lower, 2 higher
            int leaves = 0;
            for (int a = tid; a < n; a += nthr) {
                if (!flags_valid) flags[a] = is_out_box(g, in.x[a], in.y[a], in.z[a]);
                const uint32_t f = flags[a];
                cls[a] = (f & lowf[d]) ? 1 : ((f & highf[d]) ? 2 : 0);
                leaves |= cls[a];
            }
            flags_valid = true;
            // nobody crosses this dimension's faces (the usual case): the stable partition below
            // would rewrite the list unchanged
            if (!__syncthreads_or(leaves)) continue;
            int base = 0;
            for (int which = 0; which < 3; which++) {
                for (int c0 = 0; c0 < n; c0 += nthr) {
                    const int a = c0 + tid;
                    const int sel = (a < n && cls[a] == which) ? 1 : 0;
                    int ex;
                    const int tot = block_exclusive_scan(sel, ex);
                    if (sel) {
                        const int dst = base + ex;
                        inter_save(in, a, dst);
                        if (which != 0) {
                            double *rec = in.scratch_d + 13 * dst;
                            const double sh = (which == 1) ? g.L[d] : -g.L[d];
                            rec[d] = __dadd_rn(rec[d], sh);
                            rec[6] = 0.0; rec[7] = 0.0; rec[8] = 0.0; rec[9] = 0.0; rec[10] = 0.0;
                        }
                    }
                    base += tot;
                }
            }
            __syncthreads();
            for (int a = tid; a < n; a += nthr) inter_restore(in, a, a);
            flags_valid = false;
            __syncthreads();
        }
    }

    if (mask & MANAGE_BORDER) {
        // Both directions of a dimension send from the same entries, so each entry's nearest site is
        // found once per dimension. With one chunk of entries (the usual case) both directions share
        // one scan: the lower direction's selections are counted in the low 16 bits of the packed
        // sums, the higher's above them. With more, the lower pass keeps both region tests in mk
        // (bit 0 the region sent LOWER, bit 1 the one sent HIGHER) for the higher pass; each thread
        // keeps the same entries in both passes, and cap + gcap ints fit in the 13 * cap doubles of
        // scratch_d.
        int *mk = reinterpret_cast<int *>(in.scratch_d);
        for (int d = 0; d < 3; d++) {
            const int n_loc = n_inter;
            const int total = n_loc + n_ghost;
            int lo[2][3], hi[2][3];
            region_fw(g, d, 0, lo[0], hi[0]);
            region_fw(g, d, 1, lo[1], hi[1]);
            if (total <= nthr) {
                double p3[3] = {0.0, 0.0, 0.0};
                int ty = 0, root = 0, m = 0;
                if (tid < total) {
                    border_entry(in, n_loc, tid, p3, ty, root);
                    m = border_regions(g, lo, hi, p3);
                }
                int ex;
                const int tot = block_exclusive_scan((m & 1) | ((m & 2) << 15), ex);
                const int base1 = min(n_ghost + (tot & 0xffff), in.gcap);
                if (m & 1) border_put(in, n_ghost + (ex & 0xffff), p3, d, g.L[d], ty, root);
                if (m & 2) border_put(in, base1 + (ex >> 16), p3, d, -g.L[d], ty, root);
                n_ghost = min(base1 + (tot >> 16), in.gcap);
                if (tid == 0) in.cnt[CNT_GHOST] = n_ghost;
                __syncthreads();
                continue;
            }
            for (int dir = 0; dir < 2; dir++) {
                const double sh = (dir == 0) ? g.L[d] : -g.L[d];
                int base = n_ghost;
                for (int c0 = 0; c0 < total; c0 += nthr) {
                    const int e = c0 + tid;
                    int sel = 0;
                    if (e < total) {
                        if (dir == 0) {
                            double p3[3];
                            int ty, root;
                            border_entry(in, n_loc, e, p3, ty, root);
                            const int m = border_regions(g, lo, hi, p3);
                            mk[e] = m;
                            sel = m & 1;
                        } else {
                            sel = (mk[e] >> 1) & 1;
                        }
                    }
                    int ex;
                    const int tot = block_exclusive_scan(sel, ex);
                    if (sel) {
                        double p3[3];
                        int ty, root;
                        border_entry(in, n_loc, e, p3, ty, root);
                        border_put(in, base + ex, p3, d, sh, ty, root);
                    }
                    base += tot;
                }
                n_ghost = base < in.gcap ? base : in.gcap;
                if (tid == 0) in.cnt[CNT_GHOST] = n_ghost;
                __syncthreads();
            }
        }
    }

    if (mask & MANAGE_INDEX) {
        const int n_loc = n_inter;
        const int n_gh = n_ghost;
        const int total = n_loc + n_gh;
        for (int e = tid; e < total; e += nthr) {
            double px, py, pz;
            int ref;
            if (e < n_loc) { px = in.x[e]; py = in.y[e]; pz = in.z[e]; ref = e; }
            else { const int q = e - n_loc; px = in.gx[q]; py = in.gy[q]; pz = in.gz[q]; ref = in.cap + q; }
            long long c[3];
            near_lat_coord(g, px, py, pz, c);
            long long key;
            if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= g.Sx || c[1] >= g.Sy || c[2] >= g.Sz) {
                set_error(in, MG_DEVERR_OUT_OF_GRID);
                key = INT_MAX;
            } else {
                key = lin(g, (int) c[0], (int) c[1], (int) c[2]);
            }
            in.bucket[e] = (key << 32) | (long long) ref;
        }
        __syncthreads();
        extern __shared__ long long sm_keys[];
        if (total <= kSortSmemKeys) block_bitonic_sort_smem(in.bucket, total, sm_keys);
        else block_bitonic_sort(in.bucket, total);
        if (tid == 0) *in.n_bucket = total;
    }
}

// the list manager sorts up to kSortSmemKeys bucket keys in dynamic shared memory
void configure_manage_kernel() {
    cudaFuncSetAttribute(k_inter_manage, cudaFuncAttributeMaxDynamicSharedMemorySize,
                         static_cast<int>(kSortSmemKeys * sizeof(long long)));
}
void launch_inter_manage(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, int mask, bool mixed) {
    k_inter_manage<<<1, kManageThreads, kSortSmemKeys * sizeof(long long), lc.stream>>>(*lc.nt, g, s, in, mask, mixed);
}

// ------------------------------------------------------------------------------------------------
// inter-atom EAM (atom::interRho / interForce, src/atom.cpp:194-284, 360-473), FP64 arithmetic.
// One warp per local inter atom sums the atom's own terms. The Newton-3 shares that the reference
// scatters into lattice atoms (and folds from ghost slots into their owners) are summed instead by
// the owners themselves, in a fixed order, so every run gives the same bits: the inter-atom pass
// lists each lattice owner it finds inside the cutoff, and an owner gather over that list adds the
// owner's inter-atom terms in offset order, then bucket order.
// ------------------------------------------------------------------------------------------------
__device__ __forceinline__ int bucket_begin(const Inter &in, int nb, int key) {
    int lo = 0, hi = nb;
    const long long want = ((long long) key) << 32;
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        if (in.bucket[mid] < want) lo = mid + 1; else hi = mid;
    }
    return lo;
}
struct InterRef {
    double x, y, z, df;
    int type;
    uint64_t id;
};
__device__ __forceinline__ InterRef inter_ref(const Inter &in, int ref) {
    InterRef r;
    if (ref < in.cap) { r.x = in.x[ref]; r.y = in.y[ref]; r.z = in.z[ref]; r.type = in.type[ref]; r.id = in.id[ref]; r.df = in.df[ref]; }
    else {
        const int q = ref - in.cap;
        r.x = in.gx[q]; r.y = in.gy[q]; r.z = in.gz[q]; r.type = in.gtype[q]; r.id = 0; r.df = in.gdf[q];
    }
    return r;
}
__device__ __forceinline__ double rho_fn(const PotTables &pt, int type, double r2) {
    int m; double p;
    locate_d(sqrt(r2), pt.inv_dr, pt.nr, m, p);
    return val_d(pt.rho_v + type * pt.nr, m, p);
}
__device__ __forceinline__ double to_force(const PotTables &pt, int ti, int tj, double r2, double dfi, double dfj) {
    const double r = sqrt(r2);
    int m; double p;
    locate_d(r, pt.inv_dr, pt.nr, m, p);
    const double rhoip = der_d(pt.rho_d + ti * pt.nr, m, p);
    const double rhojp = der_d(pt.rho_d + tj * pt.nr, m, p);
    const double zv = val_d(pt.z_v + (ti * 3 + tj) * pt.nr, m, p);
    const double zp = der_d(pt.z_d + (ti * 3 + tj) * pt.nr, m, p);
    const double recip = 1.0 / r;
    const double phi = zv * recip;
    const double phip = zp * recip - phi * recip;
    const double psip = dfi * rhojp + dfj * rhoip + phip;
    return -psip * recip;
}
__device__ __forceinline__ double pair_fn(const PotTables &pt, int ti, int tj, double r2) {
    const double r = sqrt(r2);
    int m; double p;
    locate_d(r, pt.inv_dr, pt.nr, m, p);
    return val_d(pt.z_v + (ti * 3 + tj) * pt.nr, m, p) / r;
}
__device__ __forceinline__ double lat_df(const Geom &g, const Slots &s, int sl, bool mixed) {
    return mixed ? (double) s.df32[sidx(g, sl)] : s.df[sl];
}

// kind: 0 density, 1 force, 2 energy
// One block of kInterThreads per inter atom (the lists hold a few to thousands of atoms, each with
// ~460 partner entries): the threads share the 229 lattice entries and the 229 bucket keys of the
// atom's nearest site, two each, keep partial sums, and reduce them in a fixed order (shuffles within
// a warp, then the warps in order). With a few inter atoms the pass is one chain of dependent FP64
// spline evaluations per thread, so spreading an atom over four warps instead of one cuts its
// latency. Every lattice owner with a partner inside the cutoff is listed once (touch_owner) for
// k_inter_owner, which adds the owner's share of the pair terms.
constexpr int kInterThreads = 128;
__device__ __forceinline__ double warp_sum_d(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    return v;
}
// lists a lattice owner for the owner gather: the first caller to set its bit appends it
__device__ __forceinline__ void touch_owner(Inter &in, int own) {
    const unsigned bit = 1u << (own & 31);
    if (atomicOr(&in.touch_bits[own >> 5], bit) & bit) return;
    const int q = atomicAdd(&in.cnt[CNT_TOUCHED], 1);
    if (q < in.tcap) in.touched[q] = own;
    else set_error(in, MG_DEVERR_INTER_OVERFLOW);
}
// a slot of the local box (not a ghost slot)
__device__ __forceinline__ bool is_local_slot(const Geom &g, int sl) {
    const int X = sl % g.Sx, r = sl / g.Sx, Y = r % g.Sy, Z = r / g.Sy;
    return X >= g.gx && X < g.gx + g.bx && Y >= g.gy && Y < g.gy + g.by && Z >= g.gz && Z < g.gz + g.bz;
}
template <int KIND>
__global__ void __launch_bounds__(kInterThreads) k_inter_eam(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, PotTables pt, bool mixed) {
    const int n = in.cnt[CNT_INTER];
    const int nb = *in.n_bucket;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ double red[3][kInterThreads / 32];
    for (int a = blockIdx.x; a < n; a += gridDim.x) {  // block-uniform
        const double xa = in.x[a], ya = in.y[a], za = in.z[a];
        const int ta = in.type[a];
        const uint64_t ida = in.id[a];
        const double dfa = in.df[a];
        const int near = near_index_in_sub_box(g, xa, ya, za);
        if (near < 0) continue;
        double acc = 0.0, fx = 0.0, fy = 0.0, fz = 0.0;
        // lattice partners: the nearest site's atom, then the full offsets of that site
        const int par = (near % g.Sx) & 1;
        const int nf = nt.nfull;
        for (int q = (int) threadIdx.x - 1; q < nf; q += kInterThreads) {
            const int sj = q < 0 ? near : near + (par ? nt.full[1][q] : nt.full[0][q]);
            if (sj < 0 || sj >= g.n_slots) { set_error(in, MG_DEVERR_OUT_OF_GRID); continue; }
            const int tj = s.type[sj];
            if (tj < 0) continue;
            const double dx = xa - s.x[sj], dy = ya - s.y[sj], dz = za - s.z[sj];
            const double r2 = dx * dx + dy * dy + dz * dz;
            if (!(r2 < g.rc2)) continue;
            touch_owner(in, owner_slot(g, sj));
            if (KIND == 0) {
                acc += rho_fn(pt, tj, r2);
            } else if (KIND == 1) {
                const double fp = to_force(pt, ta, tj, r2, dfa, lat_df(g, s, sj, mixed));
                fx += dx * fp; fy += dy * fp; fz += dz * fp;
            } else {
                acc += 0.5 * pair_fn(pt, ta, tj, r2);
            }
        }
        // inter partners: same-site bucket (not itself), then the buckets of the full offsets
        for (int q = (int) threadIdx.x - 1; q < nf; q += kInterThreads) {
            const int key = q < 0 ? near : near + (par ? nt.full[1][q] : nt.full[0][q]);
            for (int b = bucket_begin(in, nb, key); b < nb && (int) (in.bucket[b] >> 32) == key; b++) {
                const InterRef o = inter_ref(in, (int) (in.bucket[b] & 0xffffffffLL));
                if (q < 0 && o.id == ida) continue;
                const double dx = xa - o.x, dy = ya - o.y, dz = za - o.z;
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (!(r2 < g.rc2)) continue;
                if (KIND == 0) acc += rho_fn(pt, o.type, r2);
                else if (KIND == 1) {
                    const double fp = to_force(pt, ta, o.type, r2, dfa, o.df);
                    fx += dx * fp; fy += dy * fp; fz += dz * fp;
                } else {
                    acc += 0.5 * pair_fn(pt, ta, o.type, r2);
                }
            }
        }
        // the threads' partial sums: shuffles within each warp, then the warps' sums in warp order
        if (KIND == 1) {
            fx = warp_sum_d(fx);
            fy = warp_sum_d(fy);
            fz = warp_sum_d(fz);
            if (lane == 0) { red[0][warp] = fx; red[1][warp] = fy; red[2][warp] = fz; }
        } else {
            acc = warp_sum_d(acc);
            if (lane == 0) red[0][warp] = acc;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            acc = red[0][0]; fy = red[1][0]; fz = red[2][0];
            for (int w = 1; w < kInterThreads / 32; w++) {
                acc += red[0][w];
                if (KIND == 1) { fy += red[1][w]; fz += red[2][w]; }
            }
            fx = acc;
        }
        __syncthreads();  // red is reused by the block's next atom
        if (threadIdx.x != 0) continue;
        if (KIND == 0) {
            in.rho[a] = acc;
            int m; double p;
            locate_d(acc, pt.inv_drho, pt.nrho, m, p);
            in.df[a] = der_d(pt.F_d + ta * pt.nrho, m, p);
        } else if (KIND == 1) {
            in.fx[a] = fx; in.fy[a] = fy; in.fz[a] = fz;
        } else {
            int m; double p;
            locate_d(in.rho[a], pt.inv_drho, pt.nrho, m, p);
            in.e[a] = val_d(pt.F_v + ta * pt.nrho, m, p) + acc;
        }
    }
}
// The lattice owners' side of the inter-atom pairs. One warp per owner listed by k_inter_eam: the
// lanes walk the owner's site and its full offsets (reference order) and, per site, the bucket of
// inter atoms whose nearest site it is (local atoms, and the ghost images borderInter made of atoms
// near the far side of the box). Each pair inside the cutoff adds the term the inter atom's pass
// would have scattered, computed from the same oriented difference x_inter - x_lattice; the lanes'
// partial sums are reduced by shuffles in a fixed order and added to the owner once. Whether a ghost
// lattice slot or a ghost inter atom carries the periodic image changes only the rounding of the
// difference. A local inter atom whose nearest site is outside the box takes no part, as in the
// inter-atom pass. The last block to finish resets the list for the next pass; the bits are clear by
// then.
template <int KIND>
__global__ void __launch_bounds__(128) k_inter_owner(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, PotTables pt, bool mixed,
                                                     StepParams *sp, bool kick) {
    const int n = min(in.cnt[CNT_TOUCHED], in.tcap);
    if (n == 0) return;  // nothing listed: no block writes, so no reset is due
    const int nb = *in.n_bucket;
    const int lane = threadIdx.x & 31;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); w < n; w += warps) {  // warp-uniform
        const int j = in.touched[w];
        const int tj = s.type[j];
        const double xj = s.x[j], yj = s.y[j], zj = s.z[j];
        const double dfj = KIND == 1 ? lat_df(g, s, j, mixed) : 0.0;
        const int par = (j % g.Sx) & 1;
        const int nf = nt.nfull;
        double acc = 0.0, fx = 0.0, fy = 0.0, fz = 0.0;
        if (tj >= 0) {
            for (int q = lane - 1; q < nf; q += 32) {
                const int key = q < 0 ? j : j + (par ? nt.full[1][q] : nt.full[0][q]);
                for (int b = bucket_begin(in, nb, key); b < nb && (int) (in.bucket[b] >> 32) == key; b++) {
                    const int ref = (int) (in.bucket[b] & 0xffffffffLL);
                    if (ref < in.cap && !is_local_slot(g, key)) continue;
                    const InterRef o = inter_ref(in, ref);
                    const double dx = o.x - xj, dy = o.y - yj, dz = o.z - zj;
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    if (!(r2 < g.rc2)) continue;
                    if (KIND == 0) {
                        acc += rho_fn(pt, o.type, r2);
                    } else if (KIND == 1) {
                        const double fp = to_force(pt, o.type, tj, r2, o.df, dfj);
                        fx += -dx * fp; fy += -dy * fp; fz += -dz * fp;
                    } else {
                        acc += 0.5 * pair_fn(pt, o.type, tj, r2);
                    }
                }
            }
        }
        if (KIND == 1) {
            fx = warp_sum_d(fx);
            fy = warp_sum_d(fy);
            fz = warp_sum_d(fz);
        } else {
            acc = warp_sum_d(acc);
        }
        if (lane == 0) {
            if (tj >= 0) {
                if (KIND == 0) s.rho[j] += acc;
                else if (KIND == 1) {
                    const double f0 = s.fx[j] + fx, f1 = s.fy[j] + fy, f2v = s.fz[j] + fz;
                    s.fx[j] = f0; s.fy[j] = f1; s.fz[j] = f2v;
                    if (kick) {  // the second half-kick the lattice force pass left to this owner
                        const double c = dt_inv_m_of(sp, tj);
                        const double vx = __dadd_rn(s.vx[j], __dmul_rn(c, f0));
                        const double vy = __dadd_rn(s.vy[j], __dmul_rn(c, f1));
                        const double vz = __dadd_rn(s.vz[j], __dmul_rn(c, f2v));
                        s.vx[j] = vx; s.vy[j] = vy; s.vz[j] = vz;
                        if (variable_dt(sp)) note_vmax2(sp, speed2(vx, vy, vz));
                    }
                }
                else s.e[j] += acc;
            }
            // the density pass's list stays for the force pass of the same positions (its bits tell
            // the lattice force pass which atoms to leave unkicked); the force and energy passes end it
            if (KIND != 0) atomicAnd(&in.touch_bits[j >> 5], ~(1u << (j & 31)));
        }
    }
    if (KIND == 0) return;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        if (atomicAdd(&in.cnt[CNT_TOUCH_DONE], 1) == (int) gridDim.x - 1) {
            in.cnt[CNT_TOUCHED] = 0;
            in.cnt[CNT_TOUCH_DONE] = 0;
            __threadfence();
        }
    }
}
template <int KIND>
void launch_inter_kind(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, StepParams *sp = nullptr,
                       bool kick = false) {
    k_inter_eam<KIND><<<lc.num_sms * 4, kInterThreads, 0, lc.stream>>>(*lc.nt, g, s, in, t, mixed);
    k_inter_owner<KIND><<<lc.num_sms * 4, 128, 0, lc.stream>>>(*lc.nt, g, s, in, t, mixed, sp, kick);
}
void launch_inter_rho(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed) {
    launch_inter_kind<0>(lc, g, s, in, t, mixed);
}
void launch_inter_force(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed, StepParams *sp, bool kick) {
    launch_inter_kind<1>(lc, g, s, in, t, mixed, sp, kick);
}
void launch_inter_energy(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, PotTables t, bool mixed) {
    launch_inter_kind<2>(lc, g, s, in, t, mixed);
}

// ------------------------------------------------------------------------------------------------
// far lattice atoms (farther than 0.2 a0 from their site). Rebuild from positions for states that did
// not come through atom::decide (uploads, the per-phase hooks).
// ------------------------------------------------------------------------------------------------
__global__ void k_far_clear(const __grid_constant__ NeighTables nt, Geom g, Inter in) {
    const int nf = min(in.cnt[CNT_FAR], in.fcap);
    mark_far_neighbourhoods(nt, g, in, 0, nf, 0, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}
__global__ void k_far_count_reset(Inter in) { in.cnt[CNT_FAR] = 0; }
__global__ void k_far_scan(Geom g, Slots s, Inter in) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= g.n_local) return;
    int i, j, k;
    const int sl = local_slot(g, t, i, j, k);
    if (s.type[sl] < 0) return;
    if (displaced_fp64(g, s, sl)) {
        const int q = atomicAdd(&in.cnt[CNT_FAR], 1);
        if (q < in.fcap) in.far_list[q] = sl;
        else set_error(in, MG_DEVERR_DISPLACED_OVERFLOW);
    }
}
__global__ void k_far_mark(const __grid_constant__ NeighTables nt, Geom g, Inter in) {
    const int nf = min(in.cnt[CNT_FAR], in.fcap);
    mark_far_neighbourhoods(nt, g, in, 0, nf, 1, blockIdx.x * blockDim.x + threadIdx.x, gridDim.x * blockDim.x);
}
void launch_far_clear(const LaunchCtx &lc, const Geom &g, Inter in) {
    k_far_clear<<<lc.num_sms * 4, 256, 0, lc.stream>>>(*lc.nt, g, in);
}
void launch_far_mark(const LaunchCtx &lc, const Geom &g, Inter in) {
    k_far_mark<<<lc.num_sms * 4, 256, 0, lc.stream>>>(*lc.nt, g, in);
}
void launch_far_rebuild(const LaunchCtx &lc, const Geom &g, Slots s, Inter in) {
    launch_far_clear(lc, g, in);
    k_far_count_reset<<<1, 1, 0, lc.stream>>>(in);
    const int b = 256;
    k_far_scan<<<(g.n_local + b - 1) / b, b, 0, lc.stream>>>(g, s, in);
    launch_far_mark(lc, g, in);
}

// ------------------------------------------------------------------------------------------------
// decide per chunk of planes, for the host step that overlaps its copies out with its copies in.
// With no inter atoms at the start of the step, decide (src/atom.cpp:21-84) puts every displaced atom
// into the list in scan order and then, in list order, moves each one whose nearest site is a vacant
// in-box slot into that slot. When every displaced atom's nearest site is its own slot, each is the
// only claimant of the slot it just vacated, so it goes back at once with its id, type, position and
// velocity: the step then differs from one without it only in the atom's displacement record, which
// recombination rewrites from the position, and in its far-list entry and neighbourhood marks. Those
// are made here, per chunk, before any density pass reads the neighbourhood. A displaced atom nearest
// another site (or outside the sub-box), or a full far list, voids the overlapped step instead: the
// host then runs the whole step again from its input.
// ------------------------------------------------------------------------------------------------
__global__ void k_spec_begin(Inter in) {
    in.cnt[CNT_FAR] = 0;
    in.cnt[CNT_SPEC_VOID] = 0;
}
void launch_spec_begin(const LaunchCtx &lc, Inter in) { k_spec_begin<<<1, 1, 0, lc.stream>>>(in); }

__global__ void k_spec_decide(const __grid_constant__ NeighTables nt, Geom g, Slots s, Inter in, int t0, int t1) {
    if (in.cnt[CNT_DISP_RAW] == 0) return;  // nothing displaced so far this step
    for (int t = t0 + blockIdx.x * blockDim.x + threadIdx.x; t < t1; t += gridDim.x * blockDim.x) {
        if (!in.dflag[t]) continue;
        int i, j, k;
        const int sl = local_slot(g, t, i, j, k);
        const double x = s.x[sl], y = s.y[sl], z = s.z[sl];
        if (near_index_in_sub_box(g, x, y, z) != sl) {
            atomicExch(&in.cnt[CNT_SPEC_VOID], 1);
            continue;
        }
        const int q = atomicAdd(&in.cnt[CNT_FAR], 1);
        if (q >= in.fcap) {
            atomicExch(&in.cnt[CNT_SPEC_VOID], 1);
            continue;
        }
        double xs, ys, zs;
        site_of(g, i + g.gx, j + g.gy, k + g.gz, xs, ys, zs);
        s.u4[sidx(g, sl)] = make_u4(g, x, y, z, xs, ys, zs, s.type[sl]);
        in.far_list[q] = sl;
        mark_far_neighbourhoods(nt, g, in, q, q + 1, 1, 0, 1);
    }
}
void launch_spec_decide(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, int t0, int t1) {
    if (t1 <= t0) return;
    const int b = 256, n = std::min((t1 - t0 + b - 1) / b, lc.num_sms * 4);
    k_spec_decide<<<n, b, 0, lc.stream>>>(*lc.nt, g, s, in, t0, t1);
}


// ------------------------------------------------------------------------------------------------
// setv (src/atom.cpp:475-494): one thread
// ------------------------------------------------------------------------------------------------
__global__ void k_setv(Slots s, int slot, double dir0, double dir1, double dir2, double energy) {
    const int ty = s.type[slot];
    const double m = (ty >= 0 && ty < 3) ? c_mass[ty] : 0.0;
    const double v_ = __dsqrt_rn(__ddiv_rn(__ddiv_rn(__dmul_rn(2.0, energy), m), kMvv2e));
    const double d_ = __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(dir0, dir0), __dmul_rn(dir1, dir1)), __dmul_rn(dir2, dir2)));
    s.vx[slot] = __dadd_rn(s.vx[slot], __ddiv_rn(__dmul_rn(v_, dir0), d_));
    s.vy[slot] = __dadd_rn(s.vy[slot], __ddiv_rn(__dmul_rn(v_, dir1), d_));
    s.vz[slot] = __dadd_rn(s.vz[slot], __ddiv_rn(__dmul_rn(v_, dir2), d_));
}
void launch_setv(const LaunchCtx &lc, const Geom &g, Slots s, int64_t slot, const double dir[3], double energy) {
    k_setv<<<1, 1, 0, lc.stream>>>(s, (int) slot, dir[0], dir[1], dir[2], energy);
}

// rescale (src/system_configuration.cpp:86-111): factor = sqrt(T / T_now) from the mvv reduction
__global__ void k_rescale(Geom g, Slots s, Inter in, const double *mvv, double t_set, uint64_t n_atoms) {
    const uint64_t dof = 3 * n_atoms - 3;
    const double scalar = __ddiv_rn(__dmul_rn(*mvv, kMvv2e), __dmul_rn((double) dof, kBoltz));
    const double f = __dsqrt_rn(__ddiv_rn(t_set, scalar));
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < g.n_local; t += stride) {
        int i, j, k;
        const int sl = local_slot(g, t, i, j, k);
        s.vx[sl] = __dmul_rn(s.vx[sl], f);
        s.vy[sl] = __dmul_rn(s.vy[sl], f);
        s.vz[sl] = __dmul_rn(s.vz[sl], f);
    }
    const int n = in.cnt[CNT_INTER];
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += stride) {
        in.vx[a] = __dmul_rn(in.vx[a], f);
        in.vy[a] = __dmul_rn(in.vy[a], f);
        in.vz[a] = __dmul_rn(in.vz[a], f);
    }
}
void launch_rescale(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, const double *d_mvv, double t_set,
                    uint64_t n_atoms) {
    k_rescale<<<lc.num_sms * 8, 256, 0, lc.stream>>>(g, s, in, d_mvv, t_set, n_atoms);
}

// ------------------------------------------------------------------------------------------------
// thermo reduction (deterministic: per-block partials, then one block in fixed order)
// out: [0] sum m v^2, [1..3] force sum, [4] potential energy, [5] vacancies
// ------------------------------------------------------------------------------------------------
constexpr int kThermoWords = 6;
__device__ __forceinline__ double warp_sum(double v) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
    return v;
}
__global__ void __launch_bounds__(256) k_thermo_partial(Geom g, Slots s, Inter in, bool with_energy, double *partials) {
    double acc[kThermoWords] = {0, 0, 0, 0, 0, 0};
    const int stride = gridDim.x * blockDim.x;
    for (int t = blockIdx.x * blockDim.x + threadIdx.x; t < g.n_local; t += stride) {
        int i, j, k;
        const int sl = local_slot(g, t, i, j, k);
        const int ty = s.type[sl];
        if (ty < 0) { acc[5] += 1.0; continue; }
        const double vx = s.vx[sl], vy = s.vy[sl], vz = s.vz[sl];
        acc[0] += (vx * vx + vy * vy + vz * vz) * c_mass[ty];
        acc[1] += s.fx[sl]; acc[2] += s.fy[sl]; acc[3] += s.fz[sl];
        if (with_energy) acc[4] += s.e[sl];
    }
    if (blockIdx.x == 0) {
        const int n = in.cnt[CNT_INTER];
        for (int a = threadIdx.x; a < n; a += blockDim.x) {
            const double vx = in.vx[a], vy = in.vy[a], vz = in.vz[a];
            acc[0] += (vx * vx + vy * vy + vz * vz) * c_mass[in.type[a]];
            acc[1] += in.fx[a]; acc[2] += in.fy[a]; acc[3] += in.fz[a];
            if (with_energy) acc[4] += in.e[a];
        }
    }
    __shared__ double sh[kThermoWords][8];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    for (int q = 0; q < kThermoWords; q++) {
        const double v = warp_sum(acc[q]);
        if (lane == 0) sh[q][w] = v;
    }
    __syncthreads();
    if (threadIdx.x < kThermoWords) {
        double v = 0;
        for (int q = 0; q < (int) (blockDim.x >> 5); q++) v += sh[threadIdx.x][q];
        partials[blockIdx.x * kThermoWords + threadIdx.x] = v;
    }
}
__global__ void k_thermo_final(const double *partials, int nb, double *out) {
    if (threadIdx.x < kThermoWords) {
        double v = 0;
        for (int b = 0; b < nb; b++) v += partials[b * kThermoWords + threadIdx.x];
        out[threadIdx.x] = v;
    }
}
void launch_thermo(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, bool with_energy, double *partials,
                   int n_partials, double *out) {
    k_thermo_partial<<<n_partials, 256, 0, lc.stream>>>(g, s, in, with_energy, partials);
    k_thermo_final<<<1, 32, 0, lc.stream>>>(partials, n_partials, out);
}

// ------------------------------------------------------------------------------------------------
// Wigner-Seitz mapping of arbitrary points (indexing parity checks)
// ------------------------------------------------------------------------------------------------
__global__ void k_ws_map(Geom g, const double *xyz, int64_t n, int64_t *coords, uint32_t *flags, int64_t *index) {
    const int64_t t = blockIdx.x * (int64_t) blockDim.x + threadIdx.x;
    if (t >= n) return;
    const double x = xyz[3 * t], y = xyz[3 * t + 1], z = xyz[3 * t + 2];
    long long c[3];
    near_lat_coord(g, x, y, z, c);
    coords[3 * t] = c[0]; coords[3 * t + 1] = c[1]; coords[3 * t + 2] = c[2];
    flags[t] = is_out_box(g, x, y, z);
    index[t] = near_index_in_sub_box(g, x, y, z);
}
void launch_ws_map(const LaunchCtx &lc, const Geom &g, const double *xyz, int64_t n, int64_t *coords, uint32_t *flags,
                   int64_t *index) {
    const int b = 256;
    k_ws_map<<<(unsigned) ((n + b - 1) / b), b, 0, lc.stream>>>(g, xyz, n, coords, flags, index);
}

// ------------------------------------------------------------------------------------------------
// Atom dump frames (AtomDump::dump, frontend/io/atom_dump.cpp:59-81, with the record of
// BufferedFileWriter::write, frontend/io/buffered_io.cpp:17-35): inter atoms in list order first, then
// the box's lattice atoms in k, j, i order without INVALID slots. An ordered compaction over groups of
// kDumpThreads local slots: count, one-block scan (offsets start after the inter atoms), write.
// ------------------------------------------------------------------------------------------------
static_assert(sizeof(mg_dump_record) == 72, "dump record layout (tools/dump2text/out_convert.cpp:18-25)");

__device__ __forceinline__ void put_dump_record(mg_dump_record *r, uint64_t id, uint64_t step, int type, double x,
                                                double y, double z, double vx, double vy, double vz) {
    mg_dump_record q;
    q.id = id;
    q.step = step;
    q.type = type;
    q.inter_type = 0;  // BufferedFileWriter::write sets 0 for every record
    q.pad_ = 0;
    q.x[0] = x; q.x[1] = y; q.x[2] = z;
    q.v[0] = vx; q.v[1] = vy; q.v[2] = vz;
    *r = q;
}
__global__ void __launch_bounds__(kDumpThreads) k_dump_count(Geom g, Slots s, int *group_count) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int live = 0;
    if (t < g.n_local) {
        int i, j, k;
        live = s.type[local_slot(g, t, i, j, k)] >= 0;
    }
    const int c = __syncthreads_count(live);
    if (threadIdx.x == 0) group_count[blockIdx.x] = c;
}
__global__ void __launch_bounds__(1024) k_dump_scan(Inter in, int *group_count, int ngroups, unsigned long long *count) {
    const int n_inter = min(in.cnt[CNT_INTER], in.cap);
    const int total = block_scan_counts(group_count, ngroups, n_inter);
    if (threadIdx.x == 0) *count = (unsigned long long) total;
}
__global__ void __launch_bounds__(kDumpThreads) k_dump_write(Geom g, Slots s, const int *group_offset, mg_dump_record *out,
                                                             uint64_t step) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    int sl = -1;
    if (t < g.n_local) {
        int i, j, k;
        sl = local_slot(g, t, i, j, k);
        if (s.type[sl] < 0) sl = -1;
    }
    int pos;
    block_exclusive_scan(sl >= 0 ? 1 : 0, pos);
    if (sl < 0) return;
    put_dump_record(out + group_offset[blockIdx.x] + pos, s.id[sl], step, s.type[sl], s.x[sl], s.y[sl], s.z[sl], s.vx[sl],
                    s.vy[sl], s.vz[sl]);
}
__global__ void k_dump_inter(Inter in, mg_dump_record *out, uint64_t step) {
    const int n = min(in.cnt[CNT_INTER], in.cap);
    for (int a = blockIdx.x * blockDim.x + threadIdx.x; a < n; a += gridDim.x * blockDim.x)
        put_dump_record(out + a, in.id[a], step, in.type[a], in.x[a], in.y[a], in.z[a], in.vx[a], in.vy[a], in.vz[a]);
}
void launch_dump_pack(const LaunchCtx &lc, const Geom &g, Slots s, Inter in, mg_dump_record *out,
                      unsigned long long *count, int *scratch, uint64_t step) {
    const int ngroups = dump_scratch_ints(g);
    k_dump_count<<<ngroups, kDumpThreads, 0, lc.stream>>>(g, s, scratch);
    k_dump_scan<<<1, 1024, 0, lc.stream>>>(in, scratch, ngroups, count);
    k_dump_write<<<ngroups, kDumpThreads, 0, lc.stream>>>(g, s, scratch, out, step);
    k_dump_inter<<<lc.num_sms, 256, 0, lc.stream>>>(in, out, step);
}

}  // namespace mg
