// Synthetic inputs of the benchmark configurations (host C++; every node is
// computed independently, so the bits do not depend on the thread count).  These produce the per-node stiffness
// and eigenstrain fields the reference would receive from its models and
// initial conditions:
//   - isotropic inclusion            Model::Solid::Affine::Isotropic
//                                    (src/Model/Solid/Affine/Isotropic.H:42-45)
//   - cubic Voronoi polycrystal      Model::Solid::Linear::Cubic
//                                    (src/Model/Solid/Linear/Cubic.H:26-35)
//                                    with Set::Matrix4<3,MajorMinor>::Cubic
//                                    (src/Set/Matrix4_MajorMinor.H:518-547)
//   - random spheres                 IC::Sphere-like two-phase medium
// Random numbers: std::mt19937_64, whose output sequence the C++ standard
// fixes, turned into doubles as (x >> 11) * 2^-53.
#include "../../include/agb.h"

#include <cmath>
#include <cstring>
#include <random>
#include <vector>

namespace {

struct Rng {
    std::mt19937_64 g;
    explicit Rng(uint64_t seed) : g(seed) {}
    double uniform() { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform(double lo, double hi) { return lo + (hi - lo) * uniform(); }
    // standard normal by Box-Muller on two uniforms
    double normal() {
        double u1 = uniform();
        while (u1 <= 0.0) u1 = uniform();
        const double u2 = uniform();
        return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
    }
};

const int PAIR[3][3] = {{0, 1, 2}, {1, 3, 4}, {2, 4, 5}};

int ut(int a, int b) {
    if (a > b) { int t = a; a = b; b = t; }
    return (a * 11 - a * a) / 2 + b;
}

// Haar-uniform rotation: normalised quaternion of 4 standard normals
void random_rotation(Rng& r, double R[9]) {
    double q[4];
    double n2 = 0.0;
    do {
        n2 = 0.0;
        for (int k = 0; k < 4; k++) { q[k] = r.normal(); n2 += q[k] * q[k]; }
    } while (n2 < 1e-12);
    const double inv = 1.0 / std::sqrt(n2);
    const double w = q[0] * inv, x = q[1] * inv, y = q[2] * inv, z = q[3] * inv;
    R[0] = 1 - 2 * (y * y + z * z); R[1] = 2 * (x * y - z * w);     R[2] = 2 * (x * z + y * w);
    R[3] = 2 * (x * y + z * w);     R[4] = 1 - 2 * (x * x + z * z); R[5] = 2 * (y * z - x * w);
    R[6] = 2 * (x * z - y * w);     R[7] = 2 * (y * z + x * w);     R[8] = 1 - 2 * (x * x + y * y);
}

}  // namespace

extern "C" {

// Cubic table (C11 on iiii, C44 on ijij with i != j, C12 on iijj with
// i != j, 0 elsewhere; no minor symmetrisation), rotated entrywise
// C'_pqst = R_pi R_sk C_ijkl R_qj R_tl, stored per major-minor class with the
// value of the class's last (p,q,s,t) in lexicographic order, as the
// reference's accessor-based assignment leaves it.
agb_status agb_cubic_stiffness(double C11, double C12, double C44, const double R[9], double out[21]) {
    if (!R || !out) return AGB_BAD_ARG;
    double Ct[3][3][3][3];
    for (int i = 0; i < 3; i++)
        for (int j = 0; j < 3; j++)
            for (int k = 0; k < 3; k++)
                for (int l = 0; l < 3; l++) {
                    double v = 0.0;
                    if (i == j && j == k && k == l) v = C11;
                    else if (i == k && j == l) v = C44;
                    else if (i == j && k == l) v = C12;
                    Ct[i][j][k][l] = v;
                }
    for (int p = 0; p < 3; p++)
        for (int q = 0; q < 3; q++)
            for (int s = 0; s < 3; s++)
                for (int t = 0; t < 3; t++) {
                    double acc = 0.0;
                    for (int i = 0; i < 3; i++)
                        for (int j = 0; j < 3; j++)
                            for (int k = 0; k < 3; k++)
                                for (int l = 0; l < 3; l++)
                                    acc += R[p * 3 + i] * R[s * 3 + k] * Ct[i][j][k][l] * R[q * 3 + j] * R[t * 3 + l];
                    out[ut(PAIR[p][q], PAIR[s][t])] = acc;
                }
    return AGB_OK;
}

agb_status agb_synth_uniform(uint64_t seed, int64_t n, double lo, double hi, double* out) {
    if (!out || n < 0) return AGB_BAD_ARG;
    Rng r(seed);
    for (int64_t q = 0; q < n; q++) out[q] = r.uniform(lo, hi);
    return AGB_OK;
}

agb_status agb_synth_inclusion_iso(int nx, int ny, int nz, const double dx[3], const double c[3], double radius,
                                   double lam_in, double mu_in, double lam_out, double mu_out, double eps_in,
                                   double* C, double* F0s) {
    if (!dx || !c || !C || nx < 1 || ny < 1 || nz < 1) return AGB_BAD_ARG;
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const int64_t id = i + (int64_t)nx * (j + (int64_t)ny * k);
                const double x = i * dx[0] - c[0], y = j * dx[1] - c[1], z = k * dx[2] - c[2];
                const bool in = std::sqrt(x * x + y * y + z * z) < radius;
                C[2 * id] = in ? lam_in : lam_out;
                C[2 * id + 1] = in ? mu_in : mu_out;
                if (F0s) F0s[id] = in ? eps_in : 0.0;
            }
    return AGB_OK;
}

agb_status agb_synth_voronoi_cubic(int nx, int ny, int nz, const double dx[3], int nseeds, uint64_t seed, double C11,
                                   double C12, double C44, double* C, int32_t* grain) {
    if (!dx || !C || nseeds < 1 || nx < 1 || ny < 1 || nz < 1) return AGB_BAD_ARG;
    Rng r(seed);
    const double L[3] = {(nx - 1) * dx[0], (ny - 1) * dx[1], (nz - 1) * dx[2]};
    std::vector<double> sx(nseeds), sy(nseeds), sz(nseeds);
    for (int s = 0; s < nseeds; s++) {
        sx[s] = r.uniform() * L[0];
        sy[s] = r.uniform() * L[1];
        sz[s] = r.uniform() * L[2];
    }
    std::vector<double> Cg(21 * (size_t)nseeds);
    for (int s = 0; s < nseeds; s++) {
        double R[9];
        random_rotation(r, R);
        agb_cubic_stiffness(C11, C12, C44, R, &Cg[21 * (size_t)s]);
    }
#pragma omp parallel for schedule(static)
    for (int k = 0; k < nz; k++)
        for (int j = 0; j < ny; j++)
            for (int i = 0; i < nx; i++) {
                const double x = i * dx[0], y = j * dx[1], z = k * dx[2];
                int best = 0;
                double bd = 1e300;
                for (int s = 0; s < nseeds; s++) {
                    const double ddx = x - sx[s], ddy = y - sy[s], ddz = z - sz[s];
                    const double d2 = ddx * ddx + ddy * ddy + ddz * ddz;
                    if (d2 < bd) { bd = d2; best = s; }
                }
                const int64_t id = i + (int64_t)nx * (j + (int64_t)ny * k);
                std::memcpy(C + 21 * id, &Cg[21 * (size_t)best], 21 * sizeof(double));
                if (grain) grain[id] = best;
            }
    return AGB_OK;
}

agb_status agb_synth_spheres_iso(int nx, int ny, int nz, const double dx[3], int nspheres, uint64_t seed, double rmin,
                                 double rmax, double lam_in, double mu_in, double lam_out, double mu_out, double smin,
                                 double smax, double* C, double* F0s, int* placed) {
    if (!dx || !C || nspheres < 0 || rmin < 0 || rmax < rmin || nx < 1 || ny < 1 || nz < 1) return AGB_BAD_ARG;
    Rng r(seed);
    const double L[3] = {(nx - 1) * dx[0], (ny - 1) * dx[1], (nz - 1) * dx[2]};
    struct S { double x, y, z, rad, s; };
    std::vector<S> sp;
    const int max_tries = 1000 * (nspheres + 1);
    for (int t = 0; t < max_tries && (int)sp.size() < nspheres; t++) {
        S c;
        c.x = r.uniform() * L[0];
        c.y = r.uniform() * L[1];
        c.z = r.uniform() * L[2];
        c.rad = r.uniform(rmin, rmax);
        c.s = r.uniform(smin, smax);
        bool ok = true;
        for (const S& o : sp) {
            const double ddx = c.x - o.x, ddy = c.y - o.y, ddz = c.z - o.z;
            if (ddx * ddx + ddy * ddy + ddz * ddz < (c.rad + o.rad) * (c.rad + o.rad)) { ok = false; break; }
        }
        if (ok) sp.push_back(c);
    }
    const int64_t N = (int64_t)nx * ny * nz;
    for (int64_t q = 0; q < N; q++) {
        C[2 * q] = lam_out;
        C[2 * q + 1] = mu_out;
        if (F0s) F0s[q] = 0.0;
    }
    for (const S& c : sp) {
        const int i0 = std::max(0, (int)std::floor((c.x - c.rad) / dx[0]));
        const int i1 = std::min(nx - 1, (int)std::ceil((c.x + c.rad) / dx[0]));
        const int j0 = std::max(0, (int)std::floor((c.y - c.rad) / dx[1]));
        const int j1 = std::min(ny - 1, (int)std::ceil((c.y + c.rad) / dx[1]));
        const int k0 = std::max(0, (int)std::floor((c.z - c.rad) / dx[2]));
        const int k1 = std::min(nz - 1, (int)std::ceil((c.z + c.rad) / dx[2]));
        for (int k = k0; k <= k1; k++)
            for (int j = j0; j <= j1; j++)
                for (int i = i0; i <= i1; i++) {
                    const double ddx = i * dx[0] - c.x, ddy = j * dx[1] - c.y, ddz = k * dx[2] - c.z;
                    if (ddx * ddx + ddy * ddy + ddz * ddz < c.rad * c.rad) {
                        const int64_t id = i + (int64_t)nx * (j + (int64_t)ny * k);
                        C[2 * id] = lam_in;
                        C[2 * id + 1] = mu_in;
                        if (F0s) F0s[id] = c.s;
                    }
                }
    }
    if (placed) *placed = (int)sp.size();
    return AGB_OK;
}

agb_status agb_synth_spheres_diffuse(int nx, int ny, int nz, const double dx[3], int nspheres, uint64_t seed,
                                     double rmin, double rmax, double eps, double lam_in, double mu_in, double lam_out,
                                     double mu_out, double smin, double smax, double* C, double* F0s, int* placed) {
    if (!dx || !C || nspheres < 0 || rmin < 0 || rmax < rmin || !(eps > 0) || nx < 1 || ny < 1 || nz < 1)
        return AGB_BAD_ARG;
    Rng r(seed);
    const double L[3] = {(nx - 1) * dx[0], (ny - 1) * dx[1], (nz - 1) * dx[2]};
    struct S { double x, y, z, rad, s; };
    std::vector<S> sp;
    const int max_tries = 1000 * (nspheres + 1);
    for (int t = 0; t < max_tries && (int)sp.size() < nspheres; t++) {
        S c;
        c.x = r.uniform() * L[0];
        c.y = r.uniform() * L[1];
        c.z = r.uniform() * L[2];
        c.rad = r.uniform(rmin, rmax);
        c.s = r.uniform(smin, smax);
        bool ok = true;
        for (const S& o : sp) {
            const double ddx = c.x - o.x, ddy = c.y - o.y, ddz = c.z - o.z;
            if (ddx * ddx + ddy * ddy + ddz * ddz < (c.rad + o.rad) * (c.rad + o.rad)) { ok = false; break; }
        }
        if (ok) sp.push_back(c);
    }
    const int64_t N = (int64_t)nx * ny * nz;
    // eta (volume fraction of inclusion) accumulated in C[2q], eigenstrain in F0s
    std::vector<double> eta(N, 0.0), f0(N, 0.0);
    for (const S& c : sp) {
        // the erf profile is below 1e-9 beyond r + 3 eps
        const double ext = c.rad + 3.0 * eps;
        const int i0 = std::max(0, (int)std::floor((c.x - ext) / dx[0]));
        const int i1 = std::min(nx - 1, (int)std::ceil((c.x + ext) / dx[0]));
        const int j0 = std::max(0, (int)std::floor((c.y - ext) / dx[1]));
        const int j1 = std::min(ny - 1, (int)std::ceil((c.y + ext) / dx[1]));
        const int k0 = std::max(0, (int)std::floor((c.z - ext) / dx[2]));
        const int k1 = std::min(nz - 1, (int)std::ceil((c.z + ext) / dx[2]));
#pragma omp parallel for schedule(static)
        for (int k = k0; k <= k1; k++)
            for (int j = j0; j <= j1; j++)
                for (int i = i0; i <= i1; i++) {
                    const double ddx = i * dx[0] - c.x, ddy = j * dx[1] - c.y, ddz = k * dx[2] - c.z;
                    const double d = std::sqrt(ddx * ddx + ddy * ddy + ddz * ddz);
                    // diffuse sphere of the reference's ellipse initial condition
                    // (A = I / r^2): 0.5 - 0.5 erf((x A x - 1) / eps / |A x|)
                    const double e = d > 0 ? 0.5 - 0.5 * std::erf((d * d - c.rad * c.rad) / (eps * d)) : 1.0;
                    const int64_t id = i + (int64_t)nx * (j + (int64_t)ny * k);
                    eta[id] += e;
                    f0[id] += e * c.s;
                }
    }
#pragma omp parallel for schedule(static)
    for (int64_t q = 0; q < N; q++) {
        const double e = std::min(1.0, std::max(0.0, eta[q]));
        C[2 * q] = (1.0 - e) * lam_out + e * lam_in;
        C[2 * q + 1] = (1.0 - e) * mu_out + e * mu_in;
        if (F0s) F0s[q] = f0[q];
    }
    if (placed) *placed = (int)sp.size();
    return AGB_OK;
}

}  // extern "C"
