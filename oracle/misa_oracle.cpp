// TEST INFRASTRUCTURE - NOT PART OF THE PRODUCT.
//
// CPU oracle: a single-rank restatement of MISA-MD's per-step EAM hot path. It exists to check the
// GB300 kernels (parity tests) and to be timed as the CPU baseline. Nothing in the product links it.
//
// What it restates, file by file (paths relative to the MISA-MD source tree):
//   src/atom.cpp                      decide, clearForce, computeEam, latRho, interRho, latDf,
//                                     latForce, interForce, setv
//   src/newton_motion.cpp:19-74       dt/(2m) table, firststep, secondstep
//   src/atom/neighbour_index.inl      offset tables (make, isPositiveIndex, begin/end)
//   src/atom/atom_list.{h,cpp}        slot indexing, exchangeAtomFirst/exchangeAtom
//   src/atom/inter_atom_list.cpp      exchangeInter, borderInter, makeIndex, clearGhost
//   src/lattice/{lattice.h,ws_utils.cpp,box.h}   BCC index math, Wigner-Seitz mapping, box flags
//   src/pack/*.cpp                    halo packers, restated as the one-rank periodic self-exchange
//   src/system_configuration.cpp      mvv, kinetic energy, temperature, rescale, systemForce
//
// libcomm v0.3.3 (absent from the tree) semantics assumed here, on one rank:
//   * BccDomain fields: sub-box = phase space / grid (integer split), ghost = setGhostSize,
//     doubled-x "dbx_" fields, meas_global_length = phase_space * lattice_const.
//   * fwCommLocalRegion(d, dir) = the mirror of the receive regions of
//     src/pack/lat_particle_packer.cpp:65-159 (the box face of width ghost), scanned z, y, x.
//   * neiSendReceive: dimensions 0,1,2 forward (2,1,0 reverse); for each dimension both directions
//     are packed before either is received; LOWER is received before HIGHER; on one rank the
//     buffer sent in a direction is received under the same direction label.
// pot v0.1.0 (absent from the tree): setfl tables interpolated with a cubic Hermite spline whose knot
// slopes come from the 5-point (fourth-order) central difference, one-sided at the ends; lookups clamp
// to the last interval. toForce returns -(F'_i rho'_j + F'_j rho'_i + phi'_ij)/r. This is the
// published setfl/EAM scheme restated; it is not pinned by any reference test.
//
// Build with -ffp-contract=off: the source expressions are evaluated as written.

#include "misa_oracle.h"

#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <list>
#include <random>
#include <sstream>
#include <string>
#include <unordered_map>
#include <vector>

namespace {

thread_local std::string g_err;

constexpr double kBoltz = 8.617343e-5;   // src/types/pre_define.h:11
constexpr double kMvv2e = 1.0364269e-4;  // src/types/pre_define.h:18
constexpr double kFtm2v = (1.0 / kMvv2e); // src/types/pre_define.h:19
constexpr int kInvalid = -1;             // src/types/atom_types.h:27
constexpr double kNeiLatCutoff = 0.5;    // src/md_building_config.h.in:24 (LAT_CUTOFF)

// src/types/atom_types.h:17-19,42-53,61-73
double atom_mass(int type) {
    switch (type) {
        case 0: return 55.845;
        case 1: return 63.546;
        case 2: return 58.6934;
        default: return 0;
    }
}
int type_key(int type) {
    switch (type) {
        case 0: return 26;
        case 1: return 29;
        case 2: return 28;
        default: return 0;
    }
}

// box flags, src/lattice/box.h:12-20
constexpr uint32_t kInBox = 0, kXLow = 1u, kXHigh = 1u << 1, kYLow = 1u << 2, kYHigh = 1u << 3,
                   kZLow = 1u << 4, kZHigh = 1u << 5;
constexpr int64_t kIndexNotExists = -1;
const uint32_t kOutFlags[3][2] = {{kXLow, kXHigh}, {kYLow, kYHigh}, {kZLow, kZHigh}};

// ------------------------------------------------------------------------------------------------
// Domain (libcomm BccDomain restated for one sub-domain)
// ------------------------------------------------------------------------------------------------
struct Domain {
    int64_t phase_space[3];
    double a0, rcf;
    int grid_size[3], grid_coord[3];
    int ghost, cut_lattice;
    int64_t sub_size[3], sub_low[3];  // cells
    int64_t ghost_ext_low[3];         // cells
    int64_t dbx_sub_size[3], dbx_sub_low[3], dbx_ghost[3], dbx_ext[3], dbx_ghost_ext_low[3];
    double L[3];
};

Domain make_domain(const orc_domain_desc &dd) {
    Domain d{};
    d.a0 = dd.lattice_const;
    d.rcf = dd.cutoff_radius_factor;
    d.cut_lattice = static_cast<int>(std::ceil(dd.cutoff_radius_factor));
    d.ghost = dd.ghost_size > 0 ? dd.ghost_size : static_cast<int>(std::ceil(dd.cutoff_radius_factor)) + 1;
    for (int i = 0; i < 3; i++) {
        d.phase_space[i] = dd.phase_space[i];
        d.grid_size[i] = dd.grid_size[i] > 0 ? dd.grid_size[i] : 1;
        d.grid_coord[i] = dd.grid_coord[i];
        const int64_t lo = d.grid_coord[i] * d.phase_space[i] / d.grid_size[i];
        const int64_t hi = (d.grid_coord[i] + 1) * d.phase_space[i] / d.grid_size[i];
        d.sub_low[i] = lo;
        d.sub_size[i] = hi - lo;
        d.ghost_ext_low[i] = lo - d.ghost;
        const int64_t m = (i == 0) ? 2 : 1;
        d.dbx_sub_size[i] = m * d.sub_size[i];
        d.dbx_sub_low[i] = m * d.sub_low[i];
        d.dbx_ghost[i] = m * d.ghost;
        d.dbx_ext[i] = d.dbx_sub_size[i] + 2 * d.dbx_ghost[i];
        d.dbx_ghost_ext_low[i] = d.dbx_sub_low[i] - d.dbx_ghost[i];
        d.L[i] = d.phase_space[i] * d.a0;
    }
    return d;
}

// ------------------------------------------------------------------------------------------------
// Wigner-Seitz nearest BCC site (src/lattice/ws_utils.cpp:66-89). Returns doubled-x global coords.
// Octant bits pick the body-centre neighbour of the nearest cube corner; the bisector plane between
// the corner and that body centre is s.delta - 3/4 = 0 with s = +-1 per axis.
// ------------------------------------------------------------------------------------------------
inline void voronoy(double X, double Y, double Z, double lc, int64_t &cx, int64_t &cy, int64_t &cz) {
    cx = static_cast<int64_t>(std::lround(X / lc));
    cy = static_cast<int64_t>(std::lround(Y / lc));
    cz = static_cast<int64_t>(std::lround(Z / lc));
    const double dx = X / lc - cx;
    const double dy = Y / lc - cy;
    const double dz = Z / lc - cz;
    const bool bx = dx > 0, by = dy > 0, bz = dz > 0;
    cx = 2 * cx;
    const double plane = (((bx ? dx : -dx) + (by ? dy : -dy)) + (bz ? dz : -dz)) + (-3.0 / 4.0);
    if (plane >= 0.0) {
        cx += bx ? 1 : -1;
        cy += by ? 0 : -1;
        cz += bz ? 0 : -1;
    }
}

uint32_t is_out_box(const Domain &d, const double *x) {
    int64_t cx, cy, cz;
    voronoy(x[0], x[1], x[2], d.a0, cx, cy, cz);
    cx -= 2 * d.sub_low[0];
    cy -= d.sub_low[1];
    cz -= d.sub_low[2];
    uint32_t f = kInBox;
    if (cx < 0) f |= kXLow; else if (cx >= 2 * d.sub_size[0]) f |= kXHigh;
    if (cy < 0) f |= kYLow; else if (cy >= d.sub_size[1]) f |= kYHigh;
    if (cz < 0) f |= kZLow; else if (cz >= d.sub_size[2]) f |= kZHigh;
    return f;
}

void near_lat_coord(const Domain &d, const double *x, int64_t *c) {  // ghost-extended coords
    int64_t cx, cy, cz;
    voronoy(x[0], x[1], x[2], d.a0, cx, cy, cz);
    c[0] = cx - 2 * d.ghost_ext_low[0];
    c[1] = cy - d.ghost_ext_low[1];
    c[2] = cz - d.ghost_ext_low[2];
}

void near_lat_sub_box_coord(const Domain &d, const double *x, int64_t *c) {
    int64_t cx, cy, cz;
    voronoy(x[0], x[1], x[2], d.a0, cx, cy, cz);
    c[0] = cx - 2 * d.sub_low[0];
    c[1] = cy - d.sub_low[1];
    c[2] = cz - d.sub_low[2];
}

inline int64_t lin_index(const Domain &d, int64_t x, int64_t y, int64_t z) {
    return (z * d.dbx_ext[1] + y) * d.dbx_ext[0] + x;
}

int64_t find_near_lat_index_in_sub_box(const Domain &d, const double *x) {
    int64_t c[3];
    near_lat_sub_box_coord(d, x, c);
    if (c[0] < 0 || c[1] < 0 || c[2] < 0 || c[0] >= 2 * d.sub_size[0] || c[1] >= d.sub_size[1] ||
        c[2] >= d.sub_size[2]) {
        return kIndexNotExists;
    }
    return lin_index(d, c[0] + 2 * d.ghost, c[1] + d.ghost, c[2] + d.ghost);
}

// ------------------------------------------------------------------------------------------------
// Neighbour offset tables (src/atom/neighbour_index.inl:13-93)
// ------------------------------------------------------------------------------------------------
bool is_positive_index(double x, double y, double z) {
    if (z > 0) return true;
    if (z == 0) {
        if (y > 0) return true;
        if (y == 0 && x > 0) return true;
    }
    return false;
}

struct OffsetTables {
    std::vector<int64_t> full_even, full_odd, half_even, half_odd;
};

OffsetTables make_offsets(int64_t size_x, int64_t size_y, int cut_lattice, double rcf) {
    OffsetTables t;
    const double lat_factor = rcf + 2 * kNeiLatCutoff;
    const double lim = lat_factor * lat_factor;
    auto index = [&](int64_t x, int64_t y, int64_t z) { return (z * size_y + y) * size_x + x; };
    for (int odd = 0; odd < 2; odd++) {
        auto &full = odd ? t.full_odd : t.full_even;
        auto &half = odd ? t.half_odd : t.half_even;
        for (int64_t zi = -cut_lattice - 1; zi <= cut_lattice + 1; zi++) {
            for (int64_t yi = -cut_lattice - 1; yi <= cut_lattice + 1; yi++) {
                for (int64_t xi = -2 * cut_lattice - 2; xi <= 2 * cut_lattice + 2; xi++) {
                    // body-centre half step; C++ remainder keeps the sign of xi
                    const double h = ((double) (xi % 2)) / 2;
                    const double z = odd ? (double) zi - h : (double) zi + h;
                    const double y = odd ? (double) yi - h : (double) yi + h;
                    const double x = (double) xi / 2;
                    const double r = x * x + y * y + z * z;
                    if (r < lim && r > 0) {
                        const bool neg_odd = xi < 0 && xi % 2 != 0;
                        const int64_t iy = neg_odd ? (odd ? yi + 1 : yi - 1) : yi;
                        const int64_t iz = neg_odd ? (odd ? zi + 1 : zi - 1) : zi;
                        const int64_t off = index(xi, iy, iz);
                        full.push_back(off);
                        if (is_positive_index(x, y, z)) half.push_back(off);
                    }
                }
            }
        }
    }
    return t;
}

// ------------------------------------------------------------------------------------------------
// setfl potential + spline (pot v0.1.0 boundary, restated)
// ------------------------------------------------------------------------------------------------
struct Spline {
    int n = 0;
    double delta = 0, inv_delta = 0;
    std::vector<double> c0, c1, c2, c3, d0, d1, d2;

    void build(const std::vector<double> &f, double dlt) {
        n = static_cast<int>(f.size());
        delta = dlt;
        inv_delta = 1.0 / dlt;
        std::vector<double> s(n);
        s[0] = f[1] - f[0];
        s[1] = 0.5 * (f[2] - f[0]);
        s[n - 2] = 0.5 * (f[n - 1] - f[n - 3]);
        s[n - 1] = f[n - 1] - f[n - 2];
        for (int m = 2; m < n - 2; m++) {
            s[m] = ((f[m - 2] - f[m + 2]) + 8.0 * (f[m + 1] - f[m - 1])) / 12.0;
        }
        c0.assign(n, 0); c1.assign(n, 0); c2.assign(n, 0); c3.assign(n, 0);
        d0.assign(n, 0); d1.assign(n, 0); d2.assign(n, 0);
        for (int m = 0; m < n; m++) {
            c0[m] = f[m];
            c1[m] = s[m];
            if (m < n - 1) {
                c2[m] = 3.0 * (f[m + 1] - f[m]) - 2.0 * s[m] - s[m + 1];
                c3[m] = s[m] + s[m + 1] - 2.0 * (f[m + 1] - f[m]);
            }
            d0[m] = c1[m] * inv_delta;
            d1[m] = 2.0 * c2[m] * inv_delta;
            d2[m] = 3.0 * c3[m] * inv_delta;
        }
    }
    inline void locate(double x, int &m, double &p) const {
        p = x * inv_delta;
        m = static_cast<int>(p);
        if (m < 0) m = 0;
        if (m > n - 2) m = n - 2;
        p -= m;
        if (p > 1.0) p = 1.0;
    }
    double value(double x) const {
        int m; double p;
        locate(x, m, p);
        return ((c3[m] * p + c2[m]) * p + c1[m]) * p + c0[m];
    }
    double deriv(double x) const {
        int m; double p;
        locate(x, m, p);
        return (d2[m] * p + d1[m]) * p + d0[m];
    }
};

struct Potential {
    int n_ele = 0;
    std::vector<int> z;        // atomic numbers, file order
    std::vector<double> mass;
    int nrho = 0, nr = 0;
    double drho = 0, dr = 0, cutoff = 0;
    std::vector<Spline> F, rho, z2;  // z2 indexed by lower-triangle pair (i>=j): i*(i+1)/2+j

    int ele(int key) const {
        for (int i = 0; i < n_ele; i++) if (z[i] == key) return i;
        return -1;
    }
    static int pair_index(int a, int b) {
        if (a < b) std::swap(a, b);
        return a * (a + 1) / 2 + b;
    }
    double charge_density(int key, double r2) const { return rho[ele(key)].value(std::sqrt(r2)); }
    double d_embed(int key, double r) const { return F[ele(key)].deriv(r); }
    double embed(int key, double r) const { return F[ele(key)].value(r); }
    double to_force(int ki, int kj, double r2, double dfi, double dfj) const {
        const double r = std::sqrt(r2);
        const int ei = ele(ki), ej = ele(kj);
        const double rhoip = rho[ei].deriv(r);
        const double rhojp = rho[ej].deriv(r);
        const Spline &zz = z2[pair_index(ei, ej)];
        const double zv = zz.value(r);
        const double zp = zz.deriv(r);
        const double recip = 1.0 / r;
        const double phi = zv * recip;
        const double phip = zp * recip - phi * recip;
        const double psip = dfi * rhojp + dfj * rhoip + phip;
        return -psip * recip;
    }
    double pair(int ki, int kj, double r2) const {
        const double r = std::sqrt(r2);
        return z2[pair_index(ele(ki), ele(kj))].value(r) / r;
    }
};

bool read_setfl(const std::string &path, Potential &p) {
    std::ifstream in(path);
    if (!in) { g_err = "cannot open setfl file " + path; return false; }
    std::string line;
    for (int i = 0; i < 3; i++) std::getline(in, line);  // comments
    if (!std::getline(in, line)) { g_err = "setfl: missing element line"; return false; }
    {
        std::istringstream ls(line);
        ls >> p.n_ele;
        if (p.n_ele <= 0 || p.n_ele > 8) { g_err = "setfl: bad element count"; return false; }
    }
    if (!(in >> p.nrho >> p.drho >> p.nr >> p.dr >> p.cutoff)) { g_err = "setfl: bad grid line"; return false; }
    if (p.nrho < 5 || p.nr < 5) { g_err = "setfl: tables too short"; return false; }
    p.z.resize(p.n_ele); p.mass.resize(p.n_ele);
    p.F.resize(p.n_ele); p.rho.resize(p.n_ele);
    std::vector<double> buf;
    for (int e = 0; e < p.n_ele; e++) {
        double a; std::string lat;
        if (!(in >> p.z[e] >> p.mass[e] >> a >> lat)) { g_err = "setfl: bad element header"; return false; }
        buf.assign(p.nrho, 0);
        for (int i = 0; i < p.nrho; i++) if (!(in >> buf[i])) { g_err = "setfl: short F table"; return false; }
        p.F[e].build(buf, p.drho);
        buf.assign(p.nr, 0);
        for (int i = 0; i < p.nr; i++) if (!(in >> buf[i])) { g_err = "setfl: short rho table"; return false; }
        p.rho[e].build(buf, p.dr);
    }
    p.z2.resize(p.n_ele * (p.n_ele + 1) / 2);
    for (int i = 0; i < p.n_ele; i++) {
        for (int j = 0; j <= i; j++) {
            buf.assign(p.nr, 0);
            for (int k = 0; k < p.nr; k++) if (!(in >> buf[k])) { g_err = "setfl: short r*phi table"; return false; }
            p.z2[Potential::pair_index(i, j)].build(buf, p.dr);
        }
    }
    return true;
}

// ------------------------------------------------------------------------------------------------
// Simulation state
// ------------------------------------------------------------------------------------------------
struct Region {
    int64_t lo[3], hi[3];
    bool in(int64_t x, int64_t y, int64_t z) const {
        return x >= lo[0] && x < hi[0] && y >= lo[1] && y < hi[1] && z >= lo[2] && z < hi[2];
    }
};

}  // namespace

struct orc_sim {
    Domain dom;
    OffsetTables nei;
    std::vector<orc_atom> atoms;
    std::list<orc_atom> inter_list, inter_ghost;
    std::vector<orc_atom *> intersend[6], interrecv[6];
    std::vector<int64_t> sendlist[6], recvlist[6];
    std::unordered_map<int64_t, std::vector<orc_atom *>> inter_map;
    Potential pot;
    double rc = 0;
    double dt = 0;
    double dt_inv_m[3] = {0, 0, 0};
    // variable timestep (extension, not in the reference): dx_max <= 0 keeps dt fixed
    double dx_max = 0, dt_min = 0, dt_max = 0;
    std::vector<double> dt_hist;  // dt of every step taken
    double sim_time = 0;

    int64_t n_slots() const { return dom.dbx_ext[0] * dom.dbx_ext[1] * dom.dbx_ext[2]; }
    int64_t idx(int64_t x, int64_t y, int64_t z) const { return lin_index(dom, x, y, z); }
    void get3d(int64_t i, int64_t &x, int64_t &y, int64_t &z) const {
        x = i % dom.dbx_ext[0];
        i /= dom.dbx_ext[0];
        y = i % dom.dbx_ext[1];
        z = i / dom.dbx_ext[1];
    }
    const std::vector<int64_t> &table(bool half, int64_t x) const {
        const bool even = (x % 2 == 0);
        if (half) return even ? nei.half_even : nei.half_odd;
        return even ? nei.full_even : nei.full_odd;
    }
    template <class F> void foreach_sub_box(F fn) {
        const Domain &d = dom;
        for (int64_t z = d.dbx_ghost[2]; z < d.dbx_sub_size[2] + d.dbx_ghost[2]; z++)
            for (int64_t y = d.dbx_ghost[1]; y < d.dbx_sub_size[1] + d.dbx_ghost[1]; y++)
                for (int64_t x = d.dbx_ghost[0]; x < d.dbx_sub_size[0] + d.dbx_ghost[0]; x++)
                    fn(atoms[idx(x, y, z)], x, y, z);
    }

    // NewtonMotion::preComputeDtInv2m (src/newton_motion.cpp:19-28)
    void set_dt(double t) {
        dt = t;
        for (int i = 0; i < 3; i++) {
            const double m = atom_mass(i);
            const double dt_halve = 0.5 * dt * kFtm2v;
            dt_inv_m[i] = dt_halve / m;
        }
    }

    // forward-communication send region (libcomm fwCommLocalRegion, assumed: the box face of
    // width ghost, mirror of src/pack/lat_particle_packer.cpp:65-159)
    Region fw_region(int d, int dir) const {
        const auto &g = dom.dbx_ghost;
        const auto &b = dom.dbx_sub_size;
        const auto &e = dom.dbx_ext;
        Region r{};
        for (int i = 0; i < 3; i++) { r.lo[i] = 0; r.hi[i] = e[i]; }
        for (int i = d + 1; i < 3; i++) { r.lo[i] = g[i]; r.hi[i] = g[i] + b[i]; }
        if (dir == 0) { r.lo[d] = g[d]; r.hi[d] = 2 * g[d]; }
        else { r.lo[d] = b[d]; r.hi[d] = b[d] + g[d]; }
        return r;
    }
    // receive region (src/pack/lat_particle_packer.cpp:65-159)
    Region recv_region(int d, int dir) const {
        const auto &g = dom.dbx_ghost;
        const auto &b = dom.dbx_sub_size;
        const auto &e = dom.dbx_ext;
        Region r{};
        for (int i = 0; i < 3; i++) { r.lo[i] = 0; r.hi[i] = e[i]; }
        for (int i = d + 1; i < 3; i++) { r.lo[i] = g[i]; r.hi[i] = g[i] + b[i]; }
        if (dir == 0) { r.lo[d] = g[d] + b[d]; r.hi[d] = e[d]; }
        else { r.lo[d] = 0; r.hi[d] = g[d]; }
        return r;
    }
    // LatParticlePacker::setOffset on one rank (src/pack/lat_particle_packer.cpp:22-32)
    double shift(int d, int dir) const {
        double s = 0.0;
        if (dom.grid_coord[d] == 0 && dir == 0) s = dom.L[d];
        if (dom.grid_coord[d] == dom.grid_size[d] - 1 && dir == 1) s = -dom.L[d];
        return s;
    }

    // ---- lattice ghost exchange (src/atom/atom_list.cpp:25-57 + LatPacker*) ----
    void exchange_atom_first() {
        for (int i = 0; i < 6; i++) { sendlist[i].clear(); recvlist[i].clear(); }
        for (int d = 0; d < 3; d++) {
            for (int dir = 0; dir < 2; dir++) {
                const Region r = fw_region(d, dir);
                auto &sl = sendlist[2 * d + dir];
                for (int64_t z = r.lo[2]; z < r.hi[2]; z++)
                    for (int64_t y = r.lo[1]; y < r.hi[1]; y++)
                        for (int64_t x = r.lo[0]; x < r.hi[0]; x++) sl.push_back(idx(x, y, z));
                const Region q = recv_region(d, dir);
                auto &rl = recvlist[2 * d + dir];
                for (int64_t z = q.lo[2]; z < q.hi[2]; z++)
                    for (int64_t y = q.lo[1]; y < q.hi[1]; y++)
                        for (int64_t x = q.lo[0]; x < q.hi[0]; x++) rl.push_back(idx(x, y, z));
            }
        }
        exchange_atom();
    }
    void exchange_atom() {
        struct Rec { int type; double r[3]; };
        for (int d = 0; d < 3; d++) {
            std::vector<Rec> buf[2];
            for (int dir = 0; dir < 2; dir++) {
                double off[3] = {0.0, 0.0, 0.0};
                off[d] = shift(d, dir);
                const auto &sl = sendlist[2 * d + dir];
                buf[dir].resize(sl.size());
                for (size_t i = 0; i < sl.size(); i++) {
                    const orc_atom &a = atoms[sl[i]];
                    buf[dir][i].type = a.type;
                    buf[dir][i].r[0] = a.x[0] + off[0];
                    buf[dir][i].r[1] = a.x[1] + off[1];
                    buf[dir][i].r[2] = a.x[2] + off[2];
                }
            }
            for (int dir = 0; dir < 2; dir++) {
                const auto &rl = recvlist[2 * d + dir];
                for (size_t i = 0; i < rl.size(); i++) {
                    orc_atom &a = atoms[rl[i]];
                    a.type = buf[dir][i].type;
                    a.x[0] = buf[dir][i].r[0];
                    a.x[1] = buf[dir][i].r[1];
                    a.x[2] = buf[dir][i].r[2];
                }
            }
        }
    }

    // ---- reverse folds (RhoPacker / ForcePacker, src/pack/rho_packer.cpp, force_packer.cpp) ----
    template <int N, class Get, class Add> void reverse_fold(Get get, Add add) {
        for (int d = 2; d >= 0; d--) {
            std::vector<double> buf[2];
            for (int dir = 0; dir < 2; dir++) {
                const auto &rl = recvlist[2 * d + (dir == 0 ? 1 : 0)];
                buf[dir].resize(rl.size() * N);
                for (size_t i = 0; i < rl.size(); i++) get(atoms[rl[i]], &buf[dir][i * N]);
            }
            for (int dir = 0; dir < 2; dir++) {
                const auto &sl = sendlist[2 * d + (dir == 0 ? 1 : 0)];
                for (size_t i = 0; i < sl.size(); i++) add(atoms[sl[i]], &buf[dir][i * N]);
            }
        }
    }

    // ---- forward df (DfEmbedPacker, src/pack/df_embed_packer.cpp) ----
    void forward_df() {
        for (int d = 0; d < 3; d++) {
            std::vector<double> buf[2];
            for (int dir = 0; dir < 2; dir++) {
                const int index = 2 * d + dir;
                for (int64_t j : sendlist[index]) buf[dir].push_back(atoms[j].df);
                for (orc_atom *p : intersend[index]) buf[dir].push_back(p->df);
            }
            for (int dir = 0; dir < 2; dir++) {
                const int index = 2 * d + dir;
                size_t m = 0;
                for (int64_t j : recvlist[index]) atoms[j].df = buf[dir][m++];
                for (orc_atom *p : interrecv[index]) {
                    if (p == nullptr) { m++; continue; }
                    p->df = buf[dir][m++];
                }
            }
        }
    }

    // ---- inter atoms ----
    // InterAtomList::exchangeInter + InterParticlePacker (src/pack/inter_particle_packer.cpp)
    void exchange_inter() {
        for (int d = 0; d < 3; d++) {
            std::vector<orc_atom> buf[2];
            for (int dir = 0; dir < 2; dir++) {
                double off[3] = {0.0};
                off[d] = shift(d, dir);
                for (auto it = inter_list.begin(); it != inter_list.end();) {
                    if (is_out_box(dom, it->x) & kOutFlags[d][dir]) {
                        orc_atom a;
                        std::memset(&a, 0, sizeof(a));
                        a.id = it->id;
                        a.type = it->type;
                        for (int k = 0; k < 3; k++) { a.x[k] = it->x[k] + off[k]; a.v[k] = it->v[k]; }
                        buf[dir].push_back(a);
                        it = inter_list.erase(it);
                    } else {
                        ++it;
                    }
                }
            }
            for (int dir = 0; dir < 2; dir++)
                for (const orc_atom &a : buf[dir]) inter_list.push_back(a);
        }
    }
    // InterAtomList::borderInter + InterBorderPacker (src/pack/inter_border_packer.cpp)
    void border_inter() {
        for (int i = 0; i < 6; i++) { intersend[i].clear(); interrecv[i].clear(); }
        for (int d = 0; d < 3; d++) {
            std::vector<orc_atom> buf[2];
            for (int dir = 0; dir < 2; dir++) {
                const int index = 2 * d + dir;
                const Region r = fw_region(d, dir);
                int64_t c[3];
                for (orc_atom &a : inter_list) {
                    near_lat_coord(dom, a.x, c);
                    if (r.in(c[0], c[1], c[2])) intersend[index].push_back(&a);
                }
                for (orc_atom &a : inter_ghost) {
                    near_lat_coord(dom, a.x, c);
                    if (r.in(c[0], c[1], c[2])) intersend[index].push_back(&a);
                }
                const double s = shift(d, dir);
                for (orc_atom *p : intersend[index]) {
                    orc_atom g;
                    std::memset(&g, 0, sizeof(g));
                    g.type = p->type;
                    for (int k = 0; k < 3; k++) g.x[k] = p->x[k];
                    g.x[d] = p->x[d] + s;
                    buf[dir].push_back(g);
                }
            }
            for (int dir = 0; dir < 2; dir++) {
                const int index = 2 * d + dir;
                for (const orc_atom &g : buf[dir]) {
                    inter_ghost.push_back(g);
                    interrecv[index].push_back(&inter_ghost.back());
                }
            }
        }
    }
    // InterAtomList::makeIndex (src/atom/inter_atom_list.cpp:27-45). Buckets keep insertion order.
    void make_index() {
        inter_map.clear();
        int64_t c[3];
        for (orc_atom &a : inter_list) {
            near_lat_coord(dom, a.x, c);
            inter_map[idx(c[0], c[1], c[2])].push_back(&a);
        }
        for (orc_atom &a : inter_ghost) {
            near_lat_coord(dom, a.x, c);
            inter_map[idx(c[0], c[1], c[2])].push_back(&a);
        }
    }
    const std::vector<orc_atom *> *bucket(int64_t key) const {
        auto it = inter_map.find(key);
        return it == inter_map.end() ? nullptr : &it->second;
    }

    // ---- atom::decide (src/atom.cpp:21-84) ----
    int decide() {
        inter_ghost.clear();
        int nflag = 0;
        const Domain &d = dom;
        const double thr = std::pow(0.2 * d.a0, 2.0);
        for (int64_t k = 0; k < d.dbx_sub_size[2]; k++) {
            for (int64_t j = 0; j < d.dbx_sub_size[1]; j++) {
                for (int64_t i = 0; i < d.dbx_sub_size[0]; i++) {
                    orc_atom &a = atoms[idx(d.dbx_ghost[0] + i, d.dbx_ghost[1] + j, d.dbx_ghost[2] + k)];
                    if (a.type == kInvalid) continue;
                    const double xt = (i + d.dbx_sub_low[0]) * 0.5 * d.a0;
                    const double yt = (j + d.dbx_sub_low[1] + (i % 2) * 0.5) * d.a0;
                    const double zt = (k + d.dbx_sub_low[2] + (i % 2) * 0.5) * d.a0;
                    double dist = (a.x[0] - xt) * (a.x[0] - xt);
                    dist += (a.x[1] - yt) * (a.x[1] - yt);
                    dist += (a.x[2] - zt) * (a.x[2] - zt);
                    if (dist > thr) {
                        inter_list.push_back(a);
                        a.type = kInvalid;
                        a.v[0] = 0; a.v[1] = 0; a.v[2] = 0;
                        nflag = 1;
                    }
                }
            }
        }
        for (auto it = inter_list.begin(); it != inter_list.end();) {
            const int64_t near = find_near_lat_index_in_sub_box(dom, it->x);
            orc_atom *n = near == kIndexNotExists ? nullptr : &atoms[near];
            if (n != nullptr && n->type == kInvalid && is_out_box(dom, n->x) == kInBox) {
                n->id = it->id;
                n->type = it->type;
                for (int c = 0; c < 3; c++) { n->x[c] = it->x[c]; n->v[c] = it->v[c]; }
                it = inter_list.erase(it);
            } else {
                ++it;
            }
        }
        return nflag;
    }

    void clear_force() {
        for (orc_atom &a : atoms) { a.f[0] = 0; a.f[1] = 0; a.f[2] = 0; a.rho = 0; }
        for (orc_atom &a : inter_list) { a.f[0] = 0; a.f[1] = 0; a.f[2] = 0; a.rho = 0; }
    }

    // ---- EAM (src/atom.cpp:102-473) ----
    void lat_rho() {
        const Domain &d = dom;
        const double rc2 = rc * rc;
        for (int64_t k = d.dbx_ghost[2]; k < d.dbx_sub_size[2] + d.dbx_ghost[2]; k++)
            for (int64_t j = d.dbx_ghost[1]; j < d.dbx_sub_size[1] + d.dbx_ghost[1]; j++)
                for (int64_t i = d.dbx_ghost[0]; i < d.dbx_sub_size[0] + d.dbx_ghost[0]; i++) {
                    const int64_t ci = idx(i, j, k);
                    orc_atom &c = atoms[ci];
                    if (c.type == kInvalid) continue;
                    for (int64_t o : table(true, i)) {
                        orc_atom &n = atoms[ci + o];
                        if (n.type == kInvalid) continue;
                        const double dx = c.x[0] - n.x[0], dy = c.x[1] - n.x[1], dz = c.x[2] - n.x[2];
                        const double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 < rc2) {
                            c.rho += pot.charge_density(type_key(n.type), r2);
                            n.rho += pot.charge_density(type_key(c.type), r2);
                        }
                    }
                }
    }
    void inter_rho() {
        const double rc2 = rc * rc;
        for (orc_atom &I : inter_list) {
            const int64_t near = find_near_lat_index_in_sub_box(dom, I.x);
            if (near == kIndexNotExists) continue;
            orc_atom &S = atoms[near];
            {
                const double dx = I.x[0] - S.x[0], dy = I.x[1] - S.x[1], dz = I.x[2] - S.x[2];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (S.type != kInvalid && r2 < rc2) {
                    I.rho += pot.charge_density(type_key(S.type), r2);
                    S.rho += pot.charge_density(type_key(I.type), r2);
                }
            }
            int64_t x, y, z;
            get3d(near, x, y, z);
            const auto &full = table(false, x);
            for (int64_t o : full) {
                orc_atom &n = atoms[near + o];
                if (n.type == kInvalid) continue;
                const double dx = I.x[0] - n.x[0], dy = I.x[1] - n.x[1], dz = I.x[2] - n.x[2];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2) {
                    I.rho += pot.charge_density(type_key(n.type), r2);
                    n.rho += pot.charge_density(type_key(I.type), r2);
                }
            }
            if (const auto *b = bucket(near)) {
                for (orc_atom *p : *b) {
                    if (p->id == I.id) continue;
                    const double dx = I.x[0] - p->x[0], dy = I.x[1] - p->x[1], dz = I.x[2] - p->x[2];
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 < rc2) I.rho += pot.charge_density(type_key(p->type), r2);
                }
            }
            for (int64_t o : full) {
                if (const auto *b = bucket(near + o)) {
                    for (orc_atom *p : *b) {
                        const double dx = I.x[0] - p->x[0], dy = I.x[1] - p->x[1], dz = I.x[2] - p->x[2];
                        const double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 < rc2) I.rho += pot.charge_density(type_key(p->type), r2);
                    }
                }
            }
            I.df = pot.d_embed(type_key(I.type), I.rho);
        }
    }
    void lat_df() {
        foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) {
            if (a.type == kInvalid) return;
            a.df = pot.d_embed(type_key(a.type), a.rho);
        });
    }
    void lat_force() {
        const Domain &d = dom;
        const double rc2 = rc * rc;
        for (int64_t k = d.dbx_ghost[2]; k < d.dbx_sub_size[2] + d.dbx_ghost[2]; k++)
            for (int64_t j = d.dbx_ghost[1]; j < d.dbx_sub_size[1] + d.dbx_ghost[1]; j++)
                for (int64_t i = d.dbx_ghost[0]; i < d.dbx_sub_size[0] + d.dbx_ghost[0]; i++) {
                    const int64_t ci = idx(i, j, k);
                    orc_atom &c = atoms[ci];
                    if (c.type == kInvalid) continue;
                    for (int64_t o : table(true, i)) {
                        orc_atom &n = atoms[ci + o];
                        const double dx = c.x[0] - n.x[0], dy = c.x[1] - n.x[1], dz = c.x[2] - n.x[2];
                        const double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 < rc2 && n.type != kInvalid) {
                            const double fp = pot.to_force(type_key(c.type), type_key(n.type), r2, c.df, n.df);
                            c.f[0] += dx * fp; c.f[1] += dy * fp; c.f[2] += dz * fp;
                            n.f[0] -= dx * fp; n.f[1] -= dy * fp; n.f[2] -= dz * fp;
                        }
                    }
                }
    }
    void inter_force() {
        const double rc2 = rc * rc;
        for (orc_atom &I : inter_list) {
            const int64_t near = find_near_lat_index_in_sub_box(dom, I.x);
            if (near == kIndexNotExists) continue;
            orc_atom &S = atoms[near];
            {
                const double dx = I.x[0] - S.x[0], dy = I.x[1] - S.x[1], dz = I.x[2] - S.x[2];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2 && S.type != kInvalid) {
                    const double fp = pot.to_force(type_key(I.type), type_key(S.type), r2, I.df, S.df);
                    I.f[0] += dx * fp; I.f[1] += dy * fp; I.f[2] += dz * fp;
                    S.f[0] -= dx * fp; S.f[1] -= dy * fp; S.f[2] -= dz * fp;
                }
            }
            int64_t x, y, z;
            get3d(near, x, y, z);
            const auto &full = table(false, x);
            for (int64_t o : full) {
                orc_atom &n = atoms[near + o];
                const double dx = I.x[0] - n.x[0], dy = I.x[1] - n.x[1], dz = I.x[2] - n.x[2];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2 && n.type != kInvalid) {
                    const double fp = pot.to_force(type_key(I.type), type_key(n.type), r2, I.df, n.df);
                    I.f[0] += dx * fp; I.f[1] += dy * fp; I.f[2] += dz * fp;
                    n.f[0] -= dx * fp; n.f[1] -= dy * fp; n.f[2] -= dz * fp;
                }
            }
            if (const auto *b = bucket(near)) {
                for (orc_atom *p : *b) {
                    if (p->id == I.id) continue;
                    const double dx = I.x[0] - p->x[0], dy = I.x[1] - p->x[1], dz = I.x[2] - p->x[2];
                    const double r2 = dx * dx + dy * dy + dz * dz;
                    if (r2 < rc2) {
                        const double fp = pot.to_force(type_key(I.type), type_key(p->type), r2, I.df, p->df);
                        I.f[0] += dx * fp; I.f[1] += dy * fp; I.f[2] += dz * fp;
                    }
                }
            }
            for (int64_t o : full) {
                if (const auto *b = bucket(near + o)) {
                    for (orc_atom *p : *b) {
                        const double dx = I.x[0] - p->x[0], dy = I.x[1] - p->x[1], dz = I.x[2] - p->x[2];
                        const double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 < rc2) {
                            const double fp = pot.to_force(type_key(I.type), type_key(p->type), r2, I.df, p->df);
                            I.f[0] += dx * fp; I.f[1] += dy * fp; I.f[2] += dz * fp;
                        }
                    }
                }
            }
        }
    }
    void compute_eam() {
        make_index();
        lat_rho();
        inter_rho();
        reverse_fold<1>([](const orc_atom &a, double *b) { b[0] = a.rho; },
                        [](orc_atom &a, const double *b) { a.rho += b[0]; });
        lat_df();
        forward_df();
        lat_force();
        inter_force();
        reverse_fold<3>([](const orc_atom &a, double *b) { b[0] = a.f[0]; b[1] = a.f[1]; b[2] = a.f[2]; },
                        [](orc_atom &a, const double *b) { a.f[0] += b[0]; a.f[1] += b[1]; a.f[2] += b[2]; });
    }

    // ---- NewtonMotion (src/newton_motion.cpp:30-74) ----
    void firststep() {
        foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) {
            if (a.type == kInvalid) return;
            const double c = dt_inv_m[a.type];
            a.v[0] = a.v[0] + c * a.f[0];
            a.v[1] = a.v[1] + c * a.f[1];
            a.v[2] = a.v[2] + c * a.f[2];
            a.x[0] += dt * a.v[0];
            a.x[1] += dt * a.v[1];
            a.x[2] += dt * a.v[2];
        });
        for (orc_atom &a : inter_list) {
            for (int d = 0; d < 3; d++) {
                a.v[d] = a.v[d] + dt_inv_m[a.type] * a.f[d];
                a.x[d] += dt * a.v[d];
            }
        }
    }
    void secondstep() {
        foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) {
            if (a.type == kInvalid) return;
            const double c = dt_inv_m[a.type];
            a.v[0] += c * a.f[0];
            a.v[1] += c * a.f[1];
            a.v[2] += c * a.f[2];
        });
        for (orc_atom &a : inter_list) {
            a.v[0] += dt_inv_m[a.type] * a.f[0];
            a.v[1] += dt_inv_m[a.type] * a.f[1];
            a.v[2] += dt_inv_m[a.type] * a.f[2];
        }
    }

    // ---- atom::setv (src/atom.cpp:475-494) ----
    void setv(const int32_t lat[4], const double dir[3], double energy) {
        const Domain &d = dom;
        if ((lat[0] * 2) >= d.dbx_sub_low[0] && (lat[0] * 2) < (d.dbx_sub_low[0] + d.dbx_sub_size[0]) &&
            lat[1] >= d.dbx_sub_low[1] && lat[1] < (d.dbx_sub_low[1] + d.dbx_sub_size[1]) &&
            lat[2] >= d.dbx_sub_low[2] && lat[2] < (d.dbx_sub_low[2] + d.dbx_sub_size[2])) {
            const int64_t kk = idx(lat[0] * 2 - d.dbx_ghost_ext_low[0], lat[1] - d.dbx_ghost_ext_low[1],
                                   lat[2] - d.dbx_ghost_ext_low[2]) + lat[3];
            orc_atom &a = atoms[kk];
            const double v_ = std::sqrt(2 * energy / atom_mass(a.type) / kMvv2e);
            const double d_ = std::sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
            a.v[0] += v_ * dir[0] / d_;
            a.v[1] += v_ * dir[1] / d_;
            a.v[2] += v_ * dir[2] / d_;
        }
    }

    // ---- system_configuration (src/system_configuration.cpp) ----
    double mvv() {
        double e = 0.0;
        foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) {
            if (a.type != kInvalid)
                e += (a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2]) * atom_mass(a.type);
        });
        for (orc_atom &a : inter_list)
            e += (a.v[0] * a.v[0] + a.v[1] * a.v[1] + a.v[2] * a.v[2]) * atom_mass(a.type);
        return e;
    }
    double temperature(uint64_t n) {
        const double t = mvv();
        const uint64_t dof = 3 * n - 3;
        return t * kMvv2e / (dof * kBoltz);
    }
    void rescale(double T, uint64_t n) {
        const double scalar = temperature(n);
        const double f = std::sqrt(T / scalar);
        foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) { a.v[0] *= f; a.v[1] *= f; a.v[2] *= f; });
        for (orc_atom &a : inter_list) { a.v[0] *= f; a.v[1] *= f; a.v[2] *= f; }
    }

    // ---- WorldBuilder::build (src/world_builder.cpp:64-199), one rank ----
    // Velocities from md_rand::random() = rand32() * (1.0 / rng.max()) of the engine the build chose
    // (src/utils/random/random.cpp:31-37, rand_generators.cpp); types from the C library's rand(),
    // which the reference leaves in its default state (srand(1) restores it here).
    template <class Engine>
    void world_build_with(Engine &rng, double rng_max, double t_set, const int32_t ratio[3]) {
        std::srand(1);
        const Domain &d = dom;
        int ratio_total = 0;
        for (int t = 0; t < 3; t++) ratio_total += ratio[t];
        uint64_t id_pre = 0;
        foreach_sub_box([&](orc_atom &a, int64_t x, int64_t y, int64_t z) {
            const int64_t i = x - d.dbx_ghost[0], j = y - d.dbx_ghost[1], k = z - d.dbx_ghost[2];
            a.id = ++id_pre;
            const int r = std::rand() % ratio_total;  // randomAtomsType
            int rank_local = 0;
            for (int t = 0; t < 3; t++) {
                rank_local += ratio[t];
                if (r < rank_local) { a.type = t; break; }
            }
            const double mass = atom_mass(a.type);
            a.x[0] = (i * 0.5) * dom.a0;
            a.x[1] = j * dom.a0 + (i % 2) * (dom.a0 / 2);
            a.x[2] = k * dom.a0 + (i % 2) * (dom.a0 / 2);
            a.v[0] = (static_cast<double>(rng()) * (1.0 / rng_max) - 0.5) / mass;
            a.v[1] = (static_cast<double>(rng()) * (1.0 / rng_max) - 0.5) / mass;
            a.v[2] = (static_cast<double>(rng()) * (1.0 / rng_max) - 0.5) / mass;
        });
        double p[4] = {0.0, 0.0, 0.0, 0.0};
        foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) {
            const double m = atom_mass(a.type);
            p[0] += a.v[0] * m;
            p[1] += a.v[1] * m;
            p[2] += a.v[2] * m;
            p[3] += m;
        });
        const uint64_t n = 2 * static_cast<uint64_t>(d.sub_size[0] * d.sub_size[1] * d.sub_size[2]);
        if (p[3] > 0.0) {
            p[0] /= n;
            p[1] /= n;
            p[2] /= n;
        }
        foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) {
            const double m = atom_mass(a.type);
            a.v[0] -= (p[0] / m);
            a.v[1] -= (p[1] / m);
            a.v[2] -= (p[2] / m);
        });
        if (t_set != 0.0) rescale(t_set, n);
    }

    // ---- per-atom potential energy (extension; follows computeEam's loop structure) ----
    double potential_energy(double *per_slot, double *per_inter, int64_t inter_cap) {
        std::vector<double> e(n_slots(), 0.0);
        std::vector<double> ei(inter_list.size(), 0.0);
        const double rc2 = rc * rc;
        const Domain &d = dom;
        foreach_sub_box([&](orc_atom &a, int64_t x, int64_t y, int64_t z) {
            if (a.type != kInvalid) e[idx(x, y, z)] += pot.embed(type_key(a.type), a.rho);
        });
        for (int64_t k = d.dbx_ghost[2]; k < d.dbx_sub_size[2] + d.dbx_ghost[2]; k++)
            for (int64_t j = d.dbx_ghost[1]; j < d.dbx_sub_size[1] + d.dbx_ghost[1]; j++)
                for (int64_t i = d.dbx_ghost[0]; i < d.dbx_sub_size[0] + d.dbx_ghost[0]; i++) {
                    const int64_t ci = idx(i, j, k);
                    const orc_atom &c = atoms[ci];
                    if (c.type == kInvalid) continue;
                    for (int64_t o : table(true, i)) {
                        const orc_atom &n = atoms[ci + o];
                        if (n.type == kInvalid) continue;
                        const double dx = c.x[0] - n.x[0], dy = c.x[1] - n.x[1], dz = c.x[2] - n.x[2];
                        const double r2 = dx * dx + dy * dy + dz * dz;
                        if (r2 < rc2) {
                            const double h = 0.5 * pot.pair(type_key(c.type), type_key(n.type), r2);
                            e[ci] += h;
                            e[ci + o] += h;
                        }
                    }
                }
        size_t ii = 0;
        for (orc_atom &I : inter_list) {
            double &eI = ei[ii++];
            eI += pot.embed(type_key(I.type), I.rho);
            const int64_t near = find_near_lat_index_in_sub_box(dom, I.x);
            if (near == kIndexNotExists) continue;
            auto lat_pair = [&](int64_t s) {
                const orc_atom &n = atoms[s];
                if (n.type == kInvalid) return;
                const double dx = I.x[0] - n.x[0], dy = I.x[1] - n.x[1], dz = I.x[2] - n.x[2];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2) {
                    const double h = 0.5 * pot.pair(type_key(I.type), type_key(n.type), r2);
                    eI += h;
                    e[s] += h;
                }
            };
            auto inter_pair = [&](const orc_atom *p) {
                const double dx = I.x[0] - p->x[0], dy = I.x[1] - p->x[1], dz = I.x[2] - p->x[2];
                const double r2 = dx * dx + dy * dy + dz * dz;
                if (r2 < rc2) eI += 0.5 * pot.pair(type_key(I.type), type_key(p->type), r2);
            };
            lat_pair(near);
            int64_t x, y, z;
            get3d(near, x, y, z);
            const auto &full = table(false, x);
            for (int64_t o : full) lat_pair(near + o);
            if (const auto *b = bucket(near))
                for (orc_atom *p : *b) if (p->id != I.id) inter_pair(p);
            for (int64_t o : full)
                if (const auto *b = bucket(near + o))
                    for (orc_atom *p : *b) inter_pair(p);
        }
        // fold ghost-slot halves into owners in the RhoPacker order
        for (int dd = 2; dd >= 0; dd--) {
            for (int dir = 0; dir < 2; dir++) {
                const auto &rl = recvlist[2 * dd + (dir == 0 ? 1 : 0)];
                const auto &sl = sendlist[2 * dd + (dir == 0 ? 1 : 0)];
                std::vector<double> buf(rl.size());
                for (size_t i = 0; i < rl.size(); i++) buf[i] = e[rl[i]];
                for (size_t i = 0; i < sl.size(); i++) e[sl[i]] += buf[i];
            }
        }
        double total = 0.0;
        foreach_sub_box([&](orc_atom &a, int64_t x, int64_t y, int64_t z) {
            const int64_t s = idx(x, y, z);
            if (a.type != kInvalid) total += e[s];
            if (per_slot) per_slot[s] = (a.type != kInvalid) ? e[s] : 0.0;
        });
        if (per_slot) {
            // zero everything outside the box
            for (int64_t s = 0; s < n_slots(); s++) {
                int64_t x, y, z;
                get3d(s, x, y, z);
                if (x < d.dbx_ghost[0] || x >= d.dbx_ghost[0] + d.dbx_sub_size[0] || y < d.dbx_ghost[1] ||
                    y >= d.dbx_ghost[1] + d.dbx_sub_size[1] || z < d.dbx_ghost[2] || z >= d.dbx_ghost[2] + d.dbx_sub_size[2])
                    per_slot[s] = 0.0;
            }
        }
        for (size_t i = 0; i < ei.size(); i++) {
            total += ei[i];
            if (per_inter && static_cast<int64_t>(i) < inter_cap) per_inter[i] = ei[i];
        }
        return total;
    }

    // dt = clamp(dx_max / max|v|, dt_min, dt_max), max over local lattice and local inter atoms of
    // (vx^2 + vy^2) + vz^2; every operation is a single IEEE rounding (built with -ffp-contract=off)
    double max_speed2() {
        double m = 0.0;
        auto note = [&](const orc_atom &a) {
            const double v2 = (a.v[0] * a.v[0] + a.v[1] * a.v[1]) + a.v[2] * a.v[2];
            if (v2 > m) m = v2;
        };
        foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) { if (a.type != kInvalid) note(a); });
        for (const orc_atom &a : inter_list) note(a);
        return m;
    }
    void step_head() {
        if (dx_max > 0) {
            const double v2 = max_speed2();
            double t = v2 > 0.0 ? dx_max / std::sqrt(v2) : dt_max;
            if (t < dt_min) t = dt_min;
            if (t > dt_max) t = dt_max;
            set_dt(t);
        }
        dt_hist.push_back(dt);
        sim_time += dt;
    }

    void step() {
        step_head();
        firststep();
        decide();
        exchange_inter();
        border_inter();
        exchange_atom();
        clear_force();
        compute_eam();
        secondstep();
    }
};

// ------------------------------------------------------------------------------------------------
// C API
// ------------------------------------------------------------------------------------------------
extern "C" {

const char *orc_last_error(void) { return g_err.c_str(); }

void orc_ws_near_lat_sub_box_coord(const orc_domain_desc *d, const double x[3], int64_t out[3]) {
    near_lat_sub_box_coord(make_domain(*d), x, out);
}
void orc_ws_near_lat_coord(const orc_domain_desc *d, const double x[3], int64_t out[3]) {
    near_lat_coord(make_domain(*d), x, out);
}
uint32_t orc_ws_is_out_box(const orc_domain_desc *d, const double x[3]) { return is_out_box(make_domain(*d), x); }
int64_t orc_ws_find_near_lat_index_in_sub_box(const orc_domain_desc *d, const double x[3]) {
    return find_near_lat_index_in_sub_box(make_domain(*d), x);
}

void orc_ws_batch(const orc_domain_desc *dd, const double *xyz, int64_t n, int64_t *ext_coords,
                  int64_t *sub_coords, uint32_t *flags, int64_t *index) {
    const Domain d = make_domain(*dd);
    for (int64_t i = 0; i < n; i++) {
        const double *x = xyz + 3 * i;
        if (ext_coords) near_lat_coord(d, x, ext_coords + 3 * i);
        if (sub_coords) near_lat_sub_box_coord(d, x, sub_coords + 3 * i);
        if (flags) flags[i] = is_out_box(d, x);
        if (index) index[i] = find_near_lat_index_in_sub_box(d, x);
    }
}

int32_t orc_nei_offsets(int64_t size_x, int64_t size_y, int64_t, int32_t cut_lattice, double rcf, int32_t which,
                        int64_t *out, int32_t cap) {
    const OffsetTables t = make_offsets(size_x, size_y, cut_lattice, rcf);
    const std::vector<int64_t> *v = which == 0 ? &t.full_even : which == 1 ? &t.full_odd
                                  : which == 2 ? &t.half_even : &t.half_odd;
    const int32_t n = static_cast<int32_t>(v->size());
    for (int32_t i = 0; i < n && i < cap; i++) out[i] = (*v)[i];
    return n;
}
int32_t orc_is_positive_index(double x, double y, double z) { return is_positive_index(x, y, z) ? 1 : 0; }

orc_sim *orc_create(const int64_t phase_space[3], double lattice_const, double rcf, const char *setfl_path,
                    double timestep_ps) {
    orc_domain_desc dd{};
    for (int i = 0; i < 3; i++) { dd.phase_space[i] = phase_space[i]; dd.grid_size[i] = 1; dd.grid_coord[i] = 0; }
    dd.lattice_const = lattice_const;
    dd.cutoff_radius_factor = rcf;
    dd.ghost_size = 0;
    auto *s = new orc_sim();
    s->dom = make_domain(dd);
    for (int i = 0; i < 3; i++) {
        if (s->dom.sub_size[i] < 2 * s->dom.ghost) {
            g_err = "box must be at least 2*ghost cells wide in every dimension";
            delete s;
            return nullptr;
        }
    }
    s->rc = s->dom.a0 * s->dom.rcf;  // atom::atom, src/atom.cpp:14-19
    s->nei = make_offsets(s->dom.dbx_ext[0], s->dom.dbx_ext[1], s->dom.cut_lattice, s->dom.rcf);
    s->atoms.assign(s->n_slots(), orc_atom{});
    for (auto &a : s->atoms) a.type = kInvalid;
    if (!read_setfl(setfl_path, s->pot)) { delete s; return nullptr; }
    s->set_dt(timestep_ps);
    return s;
}
void orc_destroy(orc_sim *s) { delete s; }

void orc_grid(const orc_sim *s, int64_t out[6]) {
    for (int i = 0; i < 3; i++) { out[i] = s->dom.dbx_ext[i]; out[3 + i] = s->dom.dbx_ghost[i]; }
}
int64_t orc_n_slots(const orc_sim *s) { return s->n_slots(); }

void orc_set_atoms(orc_sim *s, const orc_atom *atoms, int64_t n) {
    const int64_t m = std::min<int64_t>(n, s->n_slots());
    std::memcpy(s->atoms.data(), atoms, sizeof(orc_atom) * m);
}
void orc_get_atoms(const orc_sim *s, orc_atom *atoms, int64_t n) {
    const int64_t m = std::min<int64_t>(n, s->n_slots());
    std::memcpy(atoms, s->atoms.data(), sizeof(orc_atom) * m);
}
int64_t orc_get_inter(const orc_sim *s, orc_atom *out, int64_t cap) {
    int64_t i = 0;
    for (const orc_atom &a : s->inter_list) { if (i < cap) out[i] = a; i++; }
    return i;
}
int64_t orc_get_ghost_inter(const orc_sim *s, orc_atom *out, int64_t cap) {
    int64_t i = 0;
    for (const orc_atom &a : s->inter_ghost) { if (i < cap) out[i] = a; i++; }
    return i;
}
void orc_set_inter(orc_sim *s, const orc_atom *in, int64_t n) {
    s->inter_list.clear();
    for (int64_t i = 0; i < n; i++) s->inter_list.push_back(in[i]);
}
void orc_set_timestep(orc_sim *s, double dt) { s->set_dt(dt); s->dx_max = 0; }
void orc_set_variable_timestep(orc_sim *s, double dx_max, double dt_min, double dt_max) {
    s->dx_max = dx_max;
    s->dt_min = dt_min;
    s->dt_max = dt_max;
    s->set_dt(dt_max);
}
double orc_max_speed2(orc_sim *s) { return s->max_speed2(); }
int64_t orc_dt_history(const orc_sim *s, double *out, int64_t cap) {
    const int64_t n = static_cast<int64_t>(s->dt_hist.size());
    for (int64_t i = 0; i < n && i < cap; i++) out[i] = s->dt_hist[i];
    return n;
}
double orc_time(const orc_sim *s) { return s->sim_time; }

void orc_firststep(orc_sim *s) { s->firststep(); }
int32_t orc_decide(orc_sim *s) { return s->decide(); }
void orc_exchange_inter(orc_sim *s) { s->exchange_inter(); }
void orc_border_inter(orc_sim *s) { s->border_inter(); }
void orc_exchange_atom_first(orc_sim *s) { s->exchange_atom_first(); }
void orc_exchange_atom(orc_sim *s) { s->exchange_atom(); }
void orc_clear_force(orc_sim *s) { s->clear_force(); }
void orc_compute_eam(orc_sim *s) { s->compute_eam(); }
void orc_secondstep(orc_sim *s) { s->secondstep(); }

void orc_prepare(orc_sim *s) {
    s->exchange_atom_first();
    s->clear_force();
    s->compute_eam();
}
void orc_simulate(orc_sim *s, int64_t nsteps) {
    for (int64_t i = 0; i < nsteps; i++) s->step();
}
void orc_setv(orc_sim *s, const int32_t lat[4], const double dir[3], double e) { s->setv(lat, dir, e); }
void orc_collision_step(orc_sim *s, const int32_t lat[4], const double dir[3], double e) {
    s->setv(lat, dir, e);
    s->exchange_inter();
    s->border_inter();
    s->exchange_atom();
    s->clear_force();
    s->compute_eam();
}

// LegacyRand (src/utils/random/legacy_random.hpp): Park-Miller minimal standard with Schrage's method
struct OrcLegacyRand {
    int32_t s;
    uint32_t operator()() {
        const int32_t k = s / 127773;
        s = 16807 * (s - k * 127773) - 2836 * k;
        if (s < 0) s += 0x7fffffff;
        return static_cast<uint32_t>(s);
    }
};

int32_t orc_world_build(orc_sim *s, double t_set, uint32_t seed, const int32_t ratio[3], int32_t rng) {
    for (auto &a : s->atoms) { a = orc_atom{}; a.type = kInvalid; }
    s->inter_list.clear();
    switch (rng) {
        case 0: { std::mt19937 e(seed); s->world_build_with(e, static_cast<double>(std::mt19937::max()), t_set, ratio); break; }
        case 1: { std::minstd_rand e(seed); s->world_build_with(e, static_cast<double>(std::minstd_rand::max()), t_set, ratio); break; }
        case 2: { std::ranlux24 e(seed); s->world_build_with(e, static_cast<double>(std::ranlux24::max()), t_set, ratio); break; }
        case 3: { OrcLegacyRand e{static_cast<int32_t>(seed)}; s->world_build_with(e, 2147483647.0, t_set, ratio); break; }
        default: return 1;
    }
    return 0;
}

double orc_mvv(const orc_sim *s) { return const_cast<orc_sim *>(s)->mvv(); }
double orc_kinetic_energy(const orc_sim *s) { return const_cast<orc_sim *>(s)->mvv() / 2; }
double orc_temperature(const orc_sim *s, uint64_t n) { return const_cast<orc_sim *>(s)->temperature(n); }
void orc_rescale(orc_sim *s, double t, uint64_t n) { s->rescale(t, n); }
void orc_system_force(const orc_sim *s, double out[3]) {
    double fx = 0.0, fy = 0.0, fz = 0.0;
    const_cast<orc_sim *>(s)->foreach_sub_box([&](orc_atom &a, int64_t, int64_t, int64_t) {
        if (a.type != kInvalid) { fx += a.f[0]; fy += a.f[1]; fz += a.f[2]; }
    });
    for (const orc_atom &a : s->inter_list) { fx += a.f[0]; fy += a.f[1]; fz += a.f[2]; }
    out[0] = fx; out[1] = fy; out[2] = fz;
}
double orc_potential_energy(orc_sim *s, double *per_slot, double *per_inter, int64_t cap) {
    s->make_index();
    return s->potential_energy(per_slot, per_inter, cap);
}

double orc_pot_charge_density(const orc_sim *s, int32_t key, double r2) { return s->pot.charge_density(key, r2); }
double orc_pot_d_embed(const orc_sim *s, int32_t key, double rho) { return s->pot.d_embed(key, rho); }
double orc_pot_embed(const orc_sim *s, int32_t key, double rho) { return s->pot.embed(key, rho); }
double orc_pot_to_force(const orc_sim *s, int32_t ki, int32_t kj, double r2, double dfi, double dfj) {
    return s->pot.to_force(ki, kj, r2, dfi, dfj);
}
double orc_pot_pair(const orc_sim *s, int32_t ki, int32_t kj, double r2) { return s->pot.pair(ki, kj, r2); }
int32_t orc_pot_spline(const orc_sim *s, int32_t kind, int32_t e1, int32_t e2, double *out, int32_t cap) {
    const Potential &p = s->pot;
    if (e1 < 0 || e1 >= p.n_ele || e2 < 0 || e2 >= p.n_ele) return 0;
    const Spline &sp = kind == 0 ? p.F[e1] : kind == 1 ? p.rho[e1] : p.z2[Potential::pair_index(e1, e2)];
    for (int m = 0; m < sp.n && 7 * m + 6 < cap; m++) {
        out[7 * m + 0] = sp.c0[m]; out[7 * m + 1] = sp.c1[m]; out[7 * m + 2] = sp.c2[m];
        out[7 * m + 3] = sp.c3[m]; out[7 * m + 4] = sp.d0[m]; out[7 * m + 5] = sp.d1[m];
        out[7 * m + 6] = sp.d2[m];
    }
    return sp.n;
}

int64_t orc_dump_records(const orc_sim *s, uint64_t time_step, orc_dump_record *out, int64_t cap) {
    int64_t n = 0;
    auto put = [&](const orc_atom &a) {
        if (n < cap) {
            orc_dump_record &r = out[n];
            std::memset(&r, 0, sizeof(r));
            r.id = a.id;
            r.step = time_step;
            r.type = a.type;
            r.inter_type = 0;  // "normal", as the reference writes it for every atom
            for (int d = 0; d < 3; d++) { r.x[d] = a.x[d]; r.v[d] = a.v[d]; }
        }
        n++;
    };
    for (const orc_atom &a : s->inter_list) put(a);
    const Domain &d = s->dom;  // the sub-box in ghost coordinates, z outermost
    for (int64_t k = d.dbx_ghost[2]; k < d.dbx_sub_size[2] + d.dbx_ghost[2]; k++)
        for (int64_t j = d.dbx_ghost[1]; j < d.dbx_sub_size[1] + d.dbx_ghost[1]; j++)
            for (int64_t i = d.dbx_ghost[0]; i < d.dbx_sub_size[0] + d.dbx_ghost[0]; i++) {
                const orc_atom &a = s->atoms[s->idx(i, j, k)];
                if (a.type != kInvalid) put(a);
            }
    return n;
}

double orc_time_simulate(orc_sim *s, int64_t nsteps) {
    const auto t0 = std::chrono::steady_clock::now();
    for (int64_t i = 0; i < nsteps; i++) s->step();
    const auto t1 = std::chrono::steady_clock::now();
    return std::chrono::duration<double>(t1 - t0).count();
}

}  // extern "C"
