// Host side of the potential: setfl parsing and the FP64 spline coefficient build, plus the neighbour
// offset tables. This is the boundary of the external pot v0.1.0 library that MISA-MD calls
// (SetflParser / eam::interpolateFile at src/simulation.cpp:105-131); its source is not part of the
// MISA-MD tree, so the published setfl format and interpolation scheme are implemented here:
//   setfl: 3 comment lines; "N el1 .. elN"; "nrho drho nr dr cutoff"; per element "Z mass a0 lattice",
//          F(rho) on nrho knots, rho(r) on nr knots; then r*phi(r) for pairs i >= j (lower triangle).
//   spline: cubic Hermite per interval, knot slopes from the 5-point (fourth-order) central difference,
//           2- and 3-point differences at the two ends of the table. Coefficients are FP64.
// Compiled with -ffp-contract=off so every expression rounds as written.

#include <cmath>
#include <fstream>
#include <sstream>

#include "mg_internal.h"

namespace mg {

void HostSpline::build(const std::vector<double> &f, double dlt) {
    n = static_cast<int>(f.size());
    delta = dlt;
    inv_delta = 1.0 / dlt;
    std::vector<double> slope(n);
    slope[0] = f[1] - f[0];
    slope[1] = 0.5 * (f[2] - f[0]);
    slope[n - 2] = 0.5 * (f[n - 1] - f[n - 3]);
    slope[n - 1] = f[n - 1] - f[n - 2];
    for (int m = 2; m < n - 2; m++) {
        slope[m] = ((f[m - 2] - f[m + 2]) + 8.0 * (f[m + 1] - f[m - 1])) / 12.0;
    }
    c0.assign(n, 0.0); c1.assign(n, 0.0); c2.assign(n, 0.0); c3.assign(n, 0.0);
    d0.assign(n, 0.0); d1.assign(n, 0.0); d2.assign(n, 0.0);
    for (int m = 0; m < n; m++) {
        c0[m] = f[m];
        c1[m] = slope[m];
        if (m + 1 < n) {
            const double rise = f[m + 1] - f[m];
            c2[m] = 3.0 * rise - 2.0 * slope[m] - slope[m + 1];
            c3[m] = slope[m] + slope[m + 1] - 2.0 * rise;
        }
        d0[m] = c1[m] * inv_delta;
        d1[m] = 2.0 * c2[m] * inv_delta;
        d2[m] = 3.0 * c3[m] * inv_delta;
    }
}

static bool take(std::istream &in, double &v) { return static_cast<bool>(in >> v); }

bool read_setfl(const std::string &path, HostPotential &p, std::string &err) {
    std::ifstream in(path);
    if (!in) { err = "cannot open setfl file: " + path; return false; }
    std::string line;
    for (int i = 0; i < 3; i++) {
        if (!std::getline(in, line)) { err = "setfl: missing comment lines"; return false; }
    }
    if (!std::getline(in, line)) { err = "setfl: missing element line"; return false; }
    int n_ele = 0;
    {
        std::istringstream ls(line);
        if (!(ls >> n_ele) || n_ele <= 0 || n_ele > 3) { err = "setfl: element count must be 1..3"; return false; }
    }
    int nrho = 0, nr = 0;
    double drho = 0, dr = 0, cutoff = 0;
    if (!(in >> nrho >> drho >> nr >> dr >> cutoff)) { err = "setfl: bad grid line"; return false; }
    if (nrho < 5 || nr < 5 || !(drho > 0) || !(dr > 0)) { err = "setfl: bad grid values"; return false; }
    std::vector<int32_t> zs(n_ele);
    std::vector<double> F(static_cast<size_t>(n_ele) * nrho), rho(static_cast<size_t>(n_ele) * nr);
    const int n_pair = n_ele * (n_ele + 1) / 2;
    std::vector<double> rphi(static_cast<size_t>(n_pair) * nr);
    for (int e = 0; e < n_ele; e++) {
        double mass = 0, a = 0;
        std::string lattice;
        if (!(in >> zs[e] >> mass >> a >> lattice)) { err = "setfl: bad element header"; return false; }
        for (int i = 0; i < nrho; i++)
            if (!take(in, F[static_cast<size_t>(e) * nrho + i])) { err = "setfl: short F table"; return false; }
        for (int i = 0; i < nr; i++)
            if (!take(in, rho[static_cast<size_t>(e) * nr + i])) { err = "setfl: short rho table"; return false; }
    }
    for (int i = 0; i < n_ele; i++)
        for (int j = 0; j <= i; j++) {
            const int pi = HostPotential::pair_index(i, j);
            for (int k = 0; k < nr; k++)
                if (!take(in, rphi[static_cast<size_t>(pi) * nr + k])) { err = "setfl: short r*phi table"; return false; }
        }
    return build_potential(n_ele, zs.data(), nrho, drho, nr, dr, cutoff, F.data(), rho.data(), rphi.data(), p, err);
}

bool build_potential(int n_ele, const int32_t *zs, int nrho, double drho, int nr, double dr, double cutoff,
                     const double *F, const double *rho, const double *rphi, HostPotential &p, std::string &err) {
    if (n_ele <= 0 || n_ele > 3) { err = "potential: element count must be 1..3"; return false; }
    if (nrho < 5 || nr < 5 || !(drho > 0) || !(dr > 0)) { err = "potential: bad table grid"; return false; }
    p.n_ele = n_ele;
    p.z.assign(zs, zs + n_ele);
    p.nrho = nrho; p.nr = nr; p.drho = drho; p.dr = dr; p.cutoff = cutoff;
    p.F.assign(n_ele, HostSpline{});
    p.rho.assign(n_ele, HostSpline{});
    p.z2.assign(n_ele * (n_ele + 1) / 2, HostSpline{});
    std::vector<double> buf;
    for (int e = 0; e < n_ele; e++) {
        buf.assign(F + static_cast<size_t>(e) * nrho, F + static_cast<size_t>(e + 1) * nrho);
        p.F[e].build(buf, drho);
        buf.assign(rho + static_cast<size_t>(e) * nr, rho + static_cast<size_t>(e + 1) * nr);
        p.rho[e].build(buf, dr);
    }
    for (size_t q = 0; q < p.z2.size(); q++) {
        buf.assign(rphi + q * nr, rphi + (q + 1) * nr);
        p.z2[q].build(buf, dr);
    }
    return true;
}

// Offset tables. Same enumeration, radius and half-space rule as the reference so the entries come
// out in the same order; each entry also records the site-to-site vector in units of a0.
OffsetTable make_offsets(int64_t size_x, int64_t size_y, int cut_lattice, double rcf) {
    OffsetTable t;
    const double lat_factor = rcf + 2 * kNeiLatCutoff;
    const double lim = lat_factor * lat_factor;
    for (int parity = 0; parity < 2; parity++) {
        for (int64_t zi = -cut_lattice - 1; zi <= cut_lattice + 1; zi++) {
            for (int64_t yi = -cut_lattice - 1; yi <= cut_lattice + 1; yi++) {
                for (int64_t xi = -2 * cut_lattice - 2; xi <= 2 * cut_lattice + 2; xi++) {
                    const double half = ((double) (xi % 2)) / 2;
                    const double z = parity ? (double) zi - half : (double) zi + half;
                    const double y = parity ? (double) yi - half : (double) yi + half;
                    const double x = (double) xi / 2;
                    const double r = x * x + y * y + z * z;
                    if (!(r < lim && r > 0)) continue;
                    const bool wraps = xi < 0 && xi % 2 != 0;
                    const int64_t iy = wraps ? (parity ? yi + 1 : yi - 1) : yi;
                    const int64_t iz = wraps ? (parity ? zi + 1 : zi - 1) : zi;
                    const int64_t off = (iz * size_y + iy) * size_x + xi;
                    t.off[parity].push_back(off);
                    t.vec[parity].push_back(x);
                    t.vec[parity].push_back(y);
                    t.vec[parity].push_back(z);
                    const bool positive = z > 0 || (z == 0 && (y > 0 || (y == 0 && x > 0)));
                    if (positive) t.half[parity].push_back(off);
                }
            }
        }
    }
    return t;
}

}  // namespace mg
