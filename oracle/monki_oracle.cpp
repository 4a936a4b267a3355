// MONKI photon-transport oracle: a CPU FP64 restatement of the reference Fortran.
//
// TEST INFRASTRUCTURE ONLY. This file is the checker for the CUDA transport path and the
// timed CPU baseline; nothing in the product links, loads or calls it. Only tests/,
// __graft_entry__.smoke() and bench.py's cpu_baseline / --impl reference legs may use it.
//
// Parity pins: the Philox4x32-10 stream is checked against the published Random123
// known-answer vector (tests/integration/test_metal.py:43-59 of the reference); the
// transport itself has no golden output readable in this container (the archived
// goldens are NetCDF-4/HDF5 and the Fortran needs gfortran, which is absent), so its
// agreement with the Fortran is statistical, through the restated algorithm below.
//
// Restated routines (paths relative to the reference project):
//   fortran/monki/upstream/PROGRAM/mc.f90:314-1436        monte_carlo photon loop
//   fortran/monki/upstream/PROGRAM/mc.f90:1531-1580       ADVANCE_internal
//   .../modules/mc_routines_general_mod.f90:31-65          GROUND_LAMB2
//   .../modules/mc_routines_general_mod.f90:74-136         ray_scat_matrix
//   .../modules/mc_routines_general_mod.f90:147-246        ray_scat_elements / ray_scat_element
//   .../modules/mc_routines_general_mod.f90:257-480        mie_scat_matrix / mie_scat_elements
//   .../modules/mc_routines_general_mod.f90:492-670        rayl_scatter_pol
//   .../modules/mc_routines_general_mod.f90:682-932        mie_scatter_pol_bound
//   .../modules/mc_routines_general_mod.f90:942-1242       stokes_rot_mat / matmul_stokes_rot
//   .../modules/mc_routines_cartesian_mod.f90:37-393       calc_radiances_pol
//   .../modules/mc_routines_cartesian_mod.f90:849-1282     calc_radiances_and_paths_pol, ADVANCE
//   .../modules/interpol_sp.f:105-151                      linpol_dp_single
//   kernels/cpu/worker.f90:1102-1120                       transport.bin v1 layout
//   kernels/cpu/worker.f90:1126-1204                       one batch = one statistical round
//
// Deliberate differences from the Fortran, none of which changes a statistic:
//   * Random numbers come from Philox4x32-10 keyed by (seed), counter (photon, round,
//     draw block, 0), mapped to the float32 grid (w>>9 + 0.5)*2^-23 — the stream layout
//     of kernels/metal/transport.metal:64-92 — instead of gfortran RANDOM_NUMBER.
//   * Intermediates the Fortran keeps in REAL (float32) — the species cumulative sum
//     (mc.f90:1028-1036) and GROUND_LAMB2's ACOS(SQRT(P)) — are carried in FP64.
//   * Version 2 of the table stream adds one azimuth per view (the v1 stream has one);
//     version 3 adds the F34 and F44 tables of each species after F12, which the
//     reference reads from its Mie files (main_routines_general_mod.f90:790-817) but its
//     v1 export omits, so that nmat 4 (Stokes V) runs with tabulated particles.
//
// Backward transport (mc.f90:377-380, 404-415, 754-758, 790-795, 894-906, 980-982,
// 1150-1154, 1324-1336, 1393-1395; mc_routines_cartesian_mod.f90:500-520, 1034-1039):
// the photon carries the weight matrix M (identity at injection); a peel-off registers
// M P^T S0 (S0 = (1, 0, 0, 0); M As S0 at the surface) at the injection column for every
// view; the continuation sets M = M P^T (M As at the surface), samples with the Stokes
// vector (M11, M12, -M13, M14) and the + sign in the polarized sampling pdf, and divides M
// by M11; no mu0/mu factor is applied.
//   * Failure caps (history steps, detector steps, 4096 rejection attempts) report a
//     flag (1 nonfinite, 2 detector cap, 4 sampling cap, 8 invalid Stokes, 16 history
//     cap; kernels/metal/README.md:57-59) where the Fortran loops or prints.

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>
#include <stdexcept>
#include <algorithm>
#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

constexpr double kEps = 1.0e-16;
constexpr double kPi = 3.141592653589793;
constexpr double kDegToRad = 0.017453292519943295;
constexpr double kStokesCriterium = 1.0e-2;  // mc.f90 stokes_criterium_error
constexpr int kMaxAttempts = 4096;

// ---------------------------------------------------------------------------------
// Philox4x32-10 (Salmon et al. 2011, "Parallel random numbers: as easy as 1, 2, 3").
// ---------------------------------------------------------------------------------
void philox(uint32_t ctr[4], const uint32_t key_in[2]) {
    uint32_t k0 = key_in[0], k1 = key_in[1];
    for (int round = 0; round < 10; ++round) {
        uint64_t p0 = uint64_t(0xD2511F53u) * ctr[0];
        uint64_t p1 = uint64_t(0xCD9E8D57u) * ctr[2];
        uint32_t n0 = uint32_t(p1 >> 32) ^ ctr[1] ^ k0;
        uint32_t n1 = uint32_t(p1);
        uint32_t n2 = uint32_t(p0 >> 32) ^ ctr[3] ^ k1;
        uint32_t n3 = uint32_t(p0);
        ctr[0] = n0; ctr[1] = n1; ctr[2] = n2; ctr[3] = n3;
        k0 += 0x9E3779B9u;
        k1 += 0xBB67AE85u;
    }
}

// The stream of one history: counter (photon, round, block, lineage), where lineage 0 is
// the photon itself and a copy made by splitting has its own nonzero lineage.
struct Stream {
    uint32_t photon, round, seed, lineage = 0, block = 0, lane = 4, draws = 0;
    uint32_t words[4] = {0, 0, 0, 0};
    // One uniform on the open float32 grid; returned widened to double exactly.
    double uniform() {
        ++draws;
        if (lane == 4) {
            uint32_t ctr[4] = {photon, round, block++, lineage};
            uint32_t key[2] = {seed, 0};
            philox(ctr, key);
            std::memcpy(words, ctr, sizeof(words));
            lane = 0;
        }
        float u = (float(words[lane++] >> 9) + 0.5f) * 0x1p-23f;
        return double(u);
    }
};

// ---------------------------------------------------------------------------------
// Prepared tables (transport.bin v1, worker.f90:1102-1120; v2 adds per-view azimuths).
// ---------------------------------------------------------------------------------
struct Species {
    int n = 0;
    double ssalb = 0;
    std::vector<double> cosines, cdf, f11, f22, f33, f12, f34, f44;
};

struct Tables {
    int version = 0, nx = 0, ny = 0, nz = 0, nmat = 0, angles = 0, ntypes = 0;
    int k_source = 0, k_detector = 0, k_register = 0;
    bool paths = false, backward = false;
    double xunit = 0, yunit = 0, depol = 0, vartheta0 = 0, phi0 = 0, phi = 0;
    std::vector<double> zunit, vartheta, view_phi, surface, albedo, elevation;
    std::vector<double> beta, fractions, ssalb_gas;
    std::vector<Species> species;

    double beta_at(int i, int j, int k) const {  // 1-based Fortran indices
        return beta[size_t(i - 1) + size_t(nx) * (size_t(j - 1) + size_t(ny) * size_t(k - 1))];
    }
    double fraction_at(int s, int i, int j, int k) const {
        size_t cell = size_t(i - 1) + size_t(nx) * (size_t(j - 1) + size_t(ny) * size_t(k - 1));
        return fractions[size_t(s - 1) + size_t(ntypes + 1) * cell];
    }
    double zu(int k) const { return zunit[size_t(k - 1)]; }
};

Tables parse_tables(const double* raw, size_t count) {
    Tables t;
    size_t offset = 0;
    auto take = [&](size_t n) -> const double* {
        if (offset + n > count) throw std::runtime_error("Truncated transport export");
        const double* p = raw + offset;
        offset += n;
        return p;
    };
    auto as_int = [](double v, const char* what) {
        if (!std::isfinite(v) || v != std::floor(v)) throw std::runtime_error(std::string("Non-integer ") + what);
        return int(v);
    };
    if (count < 18) throw std::runtime_error("Invalid/nonfinite prepared transport export");
    for (size_t i = 0; i < count; ++i)
        if (!std::isfinite(raw[i])) throw std::runtime_error("Invalid/nonfinite prepared transport export");
    const double* h = take(12);
    t.version = as_int(h[0], "version");
    if (t.version < 1 || t.version > 3) throw std::runtime_error("Unsupported transport export version");
    t.nx = as_int(h[1], "nx"); t.ny = as_int(h[2], "ny"); t.nz = as_int(h[3], "nz");
    t.nmat = as_int(h[4], "nmat"); t.angles = as_int(h[5], "angles"); t.ntypes = as_int(h[6], "species");
    t.k_source = as_int(h[7], "k_source"); t.k_detector = as_int(h[8], "k_detector");
    t.k_register = as_int(h[9], "k_register");
    t.paths = as_int(h[10], "save_path") != 0; t.backward = as_int(h[11], "backward") != 0;
    if (t.nx < 1 || t.ny < 1 || t.nz < 2 || t.angles < 1 || t.ntypes < 0)
        throw std::runtime_error("Invalid transport export dimensions");
    if (t.nmat != 1 && t.nmat != 3 && t.nmat != 4) throw std::runtime_error("Only nmat 1, 3 or 4 is supported");
    if (t.nmat == 4 && t.version < 3 && t.ntypes > 0)
        throw std::runtime_error("nmat 4 with particles needs the version 3 table stream (F34, F44)");
    if (t.k_source != t.nz || t.k_detector != t.nz || t.k_register != t.nz)
        throw std::runtime_error("Only TOA source, detector and output grid are supported");
    const double* g = take(6);
    t.xunit = g[0]; t.yunit = g[1]; t.depol = g[2]; t.vartheta0 = g[3]; t.phi0 = g[4]; t.phi = g[5];
    const size_t cells = size_t(t.nx) * t.ny * t.nz, columns = size_t(t.nx) * t.ny;
    const double* p = take(t.nz); t.zunit.assign(p, p + t.nz);
    p = take(t.angles); t.vartheta.assign(p, p + t.angles);
    if (t.version >= 2) { p = take(t.angles); t.view_phi.assign(p, p + t.angles); }
    else t.view_phi.assign(t.angles, t.phi);
    p = take(columns); t.surface.assign(p, p + columns);
    p = take(columns); t.albedo.assign(p, p + columns);
    p = take(columns); t.elevation.assign(p, p + columns);
    p = take(cells); t.beta.assign(p, p + cells);
    p = take(cells * (t.ntypes + 1)); t.fractions.assign(p, p + cells * (t.ntypes + 1));
    p = take(t.nz); t.ssalb_gas.assign(p, p + t.nz);
    for (int s = 0; s < t.ntypes; ++s) {
        Species sp;
        const double* q = take(2);
        sp.n = as_int(q[0], "LUT size"); sp.ssalb = q[1];
        if (sp.n < 2 || sp.n > 100000) throw std::runtime_error("Invalid scattering LUT size");
        const double* c = take(size_t(sp.n) * 6);
        sp.cosines.assign(c, c + sp.n); sp.cdf.assign(c + sp.n, c + 2 * sp.n);
        sp.f11.assign(c + 2 * sp.n, c + 3 * sp.n); sp.f22.assign(c + 3 * sp.n, c + 4 * sp.n);
        sp.f33.assign(c + 4 * sp.n, c + 5 * sp.n); sp.f12.assign(c + 5 * sp.n, c + 6 * sp.n);
        if (t.version >= 3) {
            const double* v = take(size_t(sp.n) * 2);
            sp.f34.assign(v, v + sp.n); sp.f44.assign(v + sp.n, v + 2 * sp.n);
        } else {
            sp.f34.assign(size_t(sp.n), 0.0); sp.f44.assign(size_t(sp.n), 0.0);
        }
        t.species.push_back(std::move(sp));
    }
    if (offset != count) throw std::runtime_error("Trailing data in transport export");
    for (double s : t.surface) if (s != -1) throw std::runtime_error("Only Lambertian surfaces are supported");
    for (double e : t.elevation) if (e != 1) throw std::runtime_error("Only flat surfaces are supported");
    for (double z : t.zunit) if (!(z > 0)) throw std::runtime_error("Invalid layer thickness");
    for (double b : t.beta) if (b < 0) throw std::runtime_error("Negative extinction");
    for (double v : t.vartheta) if (!(v >= 0 && v < 90)) throw std::runtime_error("Viewing zenith must be in [0, 90)");
    for (const auto& sp : t.species) {
        for (int i = 1; i < sp.n; ++i)
            if (!(sp.cosines[i] > sp.cosines[i - 1])) throw std::runtime_error("Scattering cosines must increase");
        for (int i = 1; i < sp.n; ++i)
            if (sp.cdf[i] < sp.cdf[i - 1]) throw std::runtime_error("Invalid scattering CDF");
        if (std::fabs(sp.cdf[0]) > 1e-12 || std::fabs(sp.cdf[sp.n - 1] - 1) > 1e-9)
            throw std::runtime_error("Invalid scattering CDF");
    }
    return t;
}

// ---------------------------------------------------------------------------------
// Scattering helpers (mc_routines_general_mod.f90). Matrices are nmat x nmat with
// nmat <= 4, stored row-major m[r][c] with 0-based indices.
// ---------------------------------------------------------------------------------
struct Mat4 { double m[4][4]; };

// interpol_sp.f:105-151 linpol_dp_single for a two-point bracket.
double linpol2(const double x[2], const double y[2], double xp) {
    if (xp < x[0]) return (y[1] - y[0]) / (x[1] - x[0]) * (xp - x[0]) + y[0];
    if (xp > x[1]) return (y[1] - y[0]) / (x[1] - x[0]) * (xp - x[1]) + y[1];
    if (xp == x[1]) return y[1];
    if (xp == x[0]) return y[0];
    return (y[1] - y[0]) / (x[1] - x[0]) * (xp - x[0]) + y[0];
}

// mc_routines_general_mod.f90:74-136
Mat4 ray_scat_matrix(int nmat, double cs, double depol) {
    Mat4 f{};
    double sin_sca = (1.0 - cs * cs < kEps) ? 0.0 : std::sqrt(1.0 - cs * cs);
    double delta = (1.0 - depol) / (1.0 + depol / 2.0);
    double delta_prime = (1.0 - 2.0 * depol) / (1.0 - depol);
    f.m[0][0] = 3.0 / 4.0 * (1.0 + cs * cs);
    if (nmat > 1) {
        f.m[0][1] = -3.0 / 4.0 * sin_sca * sin_sca;
        f.m[1][0] = f.m[0][1];
        f.m[1][1] = 3.0 / 4.0 * (1.0 + cs * cs);
        f.m[2][2] = 3.0 / 2.0 * cs;
        if (nmat > 3) f.m[3][3] = delta_prime * f.m[2][2];
    }
    for (auto& r : f.m) for (double& v : r) v *= delta;
    f.m[0][0] += 1.0 - delta;
    for (auto& r : f.m) for (double& v : r) v /= 4.0;
    return f;
}

// mc_routines_general_mod.f90:147-197 (F11, F12)
void ray_scat_elements(double cs, double depol, double& f11, double& f12) {
    double sin_sca = (1.0 - cs * cs < kEps) ? 0.0 : std::sqrt(1.0 - cs * cs);
    double delta = (1.0 - depol) / (1.0 + depol / 2.0);
    f11 = delta * (3.0 / 4.0 * (1.0 + cs * cs)) + (1.0 - delta);
    f12 = delta * (-3.0 / 4.0 * sin_sca * sin_sca);
    f11 /= 4.0; f12 /= 4.0;
}

// mc_routines_general_mod.f90:208-246 (F11 only)
double ray_scat_element(double cs, double depol) {
    double delta = (1.0 - depol) / (1.0 + depol / 2.0);
    return (delta * (3.0 / 4.0 * (1.0 + cs * cs)) + (1.0 - delta)) / 4.0;
}

// Bracket search of mie_scat_matrix (mc_routines_general_mod.f90:296-340): an index
// guess from the uniform 0..180 degree angle grid, then a one-step correction.
int mie_bracket(const Species& sp, double cs, bool& single) {
    int n = sp.n;
    int imin = std::max(1, int((180.0 - std::acos(cs) / kDegToRad) / 180.0 * (n - 1)) + 1);
    int imax = std::min(imin + 1, n);
    single = (imax == imin);
    if (single) return imax;
    if (cs < sp.cosines[imin - 1]) imin -= 1;
    else if (cs > sp.cosines[imax - 1]) imin += 1;
    // The Fortran stops if the corrected bracket still misses; the guess relies on a
    // uniform angle grid, which the table builders here always produce.
    if (imin < 1 || imin + 1 > n || cs < sp.cosines[imin - 1] || cs > sp.cosines[imin])
        throw std::runtime_error("mie_scat_matrix: scattering cosine outside its bracket");
    return imin;
}

// mc_routines_general_mod.f90:257-388
Mat4 mie_scat_matrix(int nmat, double cs, const Species& sp) {
    Mat4 f{};
    bool single = false;
    int lo = mie_bracket(sp, cs, single);
    double f11, f22 = 0, f33 = 0, f12 = 0, f34 = 0, f44 = 0;
    if (single) {
        f11 = sp.f11[lo - 1]; f22 = sp.f22[lo - 1]; f33 = sp.f33[lo - 1]; f12 = sp.f12[lo - 1];
        f34 = sp.f34[lo - 1]; f44 = sp.f44[lo - 1];
    } else {
        const double x[2] = {sp.cosines[lo - 1], sp.cosines[lo]};
        const double y11[2] = {sp.f11[lo - 1], sp.f11[lo]}, y22[2] = {sp.f22[lo - 1], sp.f22[lo]};
        const double y33[2] = {sp.f33[lo - 1], sp.f33[lo]}, y12[2] = {sp.f12[lo - 1], sp.f12[lo]};
        const double y34[2] = {sp.f34[lo - 1], sp.f34[lo]}, y44[2] = {sp.f44[lo - 1], sp.f44[lo]};
        f11 = linpol2(x, y11, cs);
        f22 = linpol2(x, y22, cs); f33 = linpol2(x, y33, cs); f12 = linpol2(x, y12, cs);
        if (nmat > 3) { f34 = linpol2(x, y34, cs); f44 = linpol2(x, y44, cs); }
    }
    f.m[0][0] = f11;
    if (nmat > 1) { f.m[1][1] = f22; f.m[2][2] = f33; f.m[0][1] = f12; f.m[1][0] = f12; }
    if (nmat > 3) { f.m[2][3] = f34; f.m[3][2] = -f34; f.m[3][3] = f44; }
    for (auto& r : f.m) for (double& v : r) v /= 4.0;
    return f;
}

// mc_routines_general_mod.f90:400-480 (F11, F12)
void mie_scat_elements(double cs, const Species& sp, double& f11, double& f12) {
    bool single = false;
    int lo = mie_bracket(sp, cs, single);
    if (single) { f11 = sp.f11[lo - 1]; f12 = sp.f12[lo - 1]; }
    else {
        const double x[2] = {sp.cosines[lo - 1], sp.cosines[lo]};
        const double y11[2] = {sp.f11[lo - 1], sp.f11[lo]}, y12[2] = {sp.f12[lo - 1], sp.f12[lo]};
        f11 = linpol2(x, y11, cs); f12 = linpol2(x, y12, cs);
    }
    f11 /= 4.0; f12 /= 4.0;
}

double fortran_sign(double a, double b) { return std::signbit(b) ? -std::fabs(a) : std::fabs(a); }

// mc_routines_general_mod.f90:942-1174. Returns L1, L2 for nmat == 3 as the
// (C, S) pairs: L(2,2) = L(3,3) = C, L(3,2) = S, L(2,3) = -S.
struct Rotation { double c1 = 1, s1 = 0, c2 = 1, s2 = 0; };

Rotation stokes_rot_mat(double cs, double uo, double u1, double phio, double phi1, int nmat) {
    Rotation r;
    if (nmat < 3) return r;
    double dphi = std::fabs(phio - phi1);
    double rem = std::fmod(dphi, kPi);
    if (rem < kEps || std::fabs(rem - kPi) < kEps) return r;
    if (std::fabs(uo) > 1.0 - kEps && std::fabs(u1) > 1.0 - kEps) return r;
    double fac = 1.0 - uo * uo;
    double sino = fac < kEps ? 0.0 : std::sqrt(fac);
    fac = 1.0 - u1 * u1;
    double sin1 = fac < kEps ? 0.0 : std::sqrt(fac);
    double wo[3] = {sino * std::cos(phio), sino * std::sin(phio), uo};
    double w1[3] = {sin1 * std::cos(phi1), sin1 * std::sin(phi1), u1};
    double cosi1, cosi2, q;
    if (std::fabs(uo) > 1.0 - kEps || std::fabs(u1) > 1.0 - kEps) {
        double wophi[2] = {std::cos(phio), std::sin(phio)};
        double w1phi[2] = {std::cos(phi1), std::sin(phi1)};
        if (std::fabs(u1) > 1.0 - kEps) {
            cosi1 = fortran_sign(1.0, u1);
            cosi2 = -cosi1 * (w1phi[0] * wophi[0] + w1phi[1] * wophi[1]);
            q = wo[1] * w1phi[0] - wo[0] * w1phi[1];
        } else {
            cosi2 = fortran_sign(1.0, uo);
            cosi1 = -cosi2 * (w1phi[0] * wophi[0] + w1phi[1] * wophi[1]);
            q = wophi[1] * w1[0] - wophi[0] * w1[1];
        }
    } else {
        cosi1 = (u1 - uo * cs) / std::sqrt(std::max(kEps, (1.0 - uo * uo) * (1.0 - cs * cs)));
        cosi2 = (uo - u1 * cs) / std::sqrt(std::max(kEps, (1.0 - u1 * u1) * (1.0 - cs * cs)));
        q = wo[1] * w1[0] - wo[0] * w1[1];
    }
    fac = 1.0 - cosi1 * cosi1;
    double sini1 = fac < kEps ? 0.0 : std::sqrt(fac) * fortran_sign(1.0, q);
    fac = 1.0 - cosi2 * cosi2;
    double sini2 = fac < kEps ? 0.0 : std::sqrt(fac) * fortran_sign(1.0, q);
    // L(2,2) = cos^2 - sin^2 ; L(2,3) = -2 sin cos ; L(3,2) = -L(2,3)
    r.c1 = cosi1 * cosi1 - sini1 * sini1;
    r.s1 = 2.0 * sini1 * cosi1;
    r.c2 = cosi2 * cosi2 - sini2 * sini2;
    r.s2 = 2.0 * sini2 * cosi2;
    return r;
}

// mc_routines_general_mod.f90:1184-1242
Mat4 matmul_stokes_rot(int nmat, const Mat4& a, const Rotation& r) {
    Mat4 p{};
    p.m[0][0] = a.m[0][0];
    if (nmat > 1) {
        double C1 = r.c1, S1 = r.s1, C2 = r.c2, S2 = r.s2;
        p.m[0][1] = a.m[0][1] * C1;
        p.m[0][2] = -a.m[0][1] * S1;
        p.m[1][0] = C2 * a.m[1][0];
        p.m[1][1] = C1 * C2 * a.m[1][1] - S1 * S2 * a.m[2][2];
        p.m[1][2] = -C2 * S1 * a.m[1][1] - C1 * S2 * a.m[2][2];
        p.m[2][0] = S2 * a.m[1][0];
        p.m[2][1] = C1 * S2 * a.m[1][1] + C2 * S1 * a.m[2][2];
        p.m[2][2] = C1 * C2 * a.m[2][2] - S1 * S2 * a.m[1][1];
        if (nmat == 4) {
            p.m[3][1] = S1 * a.m[3][2];
            p.m[3][2] = C1 * a.m[3][2];
            p.m[3][3] = a.m[3][3];
            p.m[1][3] = -S2 * a.m[2][3];
            p.m[2][3] = C2 * a.m[2][3];
        }
    }
    return p;
}

void apply(int nmat, const Mat4& p, const double s[4], double out[4]) {
    for (int r = 0; r < nmat; ++r) {
        double acc = 0;
        for (int c = 0; c < nmat; ++c) acc += p.m[r][c] * s[c];
        out[r] = acc;
    }
}

// Spherical trigonometry shared by rayl_scatter_pol and mie_scatter_pol_bound
// (mc_routines_general_mod.f90:633-667 and :905-931).
void outgoing_direction(double cos_in, double cos_sca, double sigma1, double& cos_out, double& dphi) {
    double sin_in = std::sqrt(std::max(kEps, 1.0 - cos_in * cos_in));
    double sin_sca = std::sqrt(std::max(kEps, 1.0 - cos_sca * cos_sca));
    cos_out = cos_in * cos_sca + sin_in * sin_sca * std::cos(sigma1);
    double sin_out = std::sqrt(std::max(kEps, 1.0 - cos_out * cos_out));
    double frac = (cos_sca - cos_in * cos_out) / (sin_in * sin_out);
    if (frac >= 1.0 - kEps) dphi = 0.0;
    else if (frac <= -1.0 + kEps) dphi = kPi;
    else dphi = std::acos(frac) * fortran_sign(1.0, sigma1);
    dphi = -dphi;
}

// rayl_scatter_pol (sign -1 forward, +1 backward), with a 4096-attempt cap.
bool rayl_scatter_pol(int nmat, double depol, const double s[4], double cos_in, Stream& rng,
                      double& cos_out, double& dphi, double& cos_sca, double sign = -1.0) {
    double pdf_max = ray_scat_element(1.0, depol);
    for (int attempt = 0; attempt < kMaxAttempts; ++attempt) {
        double ran1 = rng.uniform();
        double rc = 2.0 * ran1 - 1.0;
        double ran2 = rng.uniform();
        double sigma = 2.0 * kPi * ran2 - kPi;
        double f11, f12;
        ray_scat_elements(rc, depol, f11, f12);
        if (nmat == 1) f12 = 0.0;
        double pdf = nmat == 1 ? f11 : f11 + f12 * (s[1] * std::cos(2.0 * sigma) + sign * s[2] * std::sin(2.0 * sigma));
        double ran3 = rng.uniform();
        if (ran3 * pdf_max > pdf) continue;
        cos_sca = rc;
        outgoing_direction(cos_in, cos_sca, sigma, cos_out, dphi);
        return true;
    }
    return false;
}

// mie_scatter_pol_bound (sign -1 forward, +1 backward), with a 4096-attempt cap.
bool mie_scatter_pol_bound(int nmat, const Species& sp, const double s[4], double cos_in, Stream& rng,
                           double& cos_out, double& dphi, double& cos_sca, double sign = -1.0) {
    for (int attempt = 0; attempt < kMaxAttempts; ++attempt) {
        double ran_cdf = rng.uniform();
        // Binary search of mie_scatter_pol_bound (:733-756) on 1-based indices.
        int low = 1, high = sp.n, middle = 0;
        bool found = false;
        while (low <= high && !found) {
            middle = (low + high) / 2;
            if (middle + 1 > sp.n) break;
            double v0 = sp.cdf[middle - 1], v1 = sp.cdf[middle];
            if (ran_cdf >= v0 && ran_cdf <= v1) found = true;
            else if (ran_cdf < v0) high = middle;
            else low = middle;
        }
        if (!found) throw std::runtime_error("ran_CDF not found in CDF_bound");
        const double cdf2[2] = {sp.cdf[middle - 1], sp.cdf[middle]};
        const double ang2[2] = {sp.cosines[middle - 1], sp.cosines[middle]};
        double rc = linpol2(cdf2, ang2, ran_cdf);
        double ran2 = rng.uniform();
        double sigma = 2.0 * kPi * ran2 - kPi;
        double f11, f12;
        mie_scat_elements(rc, sp, f11, f12);
        if (nmat == 1) f12 = 0.0;
        double pdf = nmat == 1 ? f11 : f11 + f12 * (s[1] * std::cos(2.0 * sigma) + sign * s[2] * std::sin(2.0 * sigma));
        double ran3 = rng.uniform();
        double bound = f11 + std::fabs(f12);
        if (ran3 * bound > pdf) continue;
        cos_sca = rc;
        outgoing_direction(cos_in, cos_sca, sigma, cos_out, dphi);
        return true;
    }
    return false;
}

// ---------------------------------------------------------------------------------
// Guided transport: detector directional importance sampling (DDIS) and Russian
// roulette, the unbiased variance reduction of Buras & Mayer (2011), "Efficient unbiased
// variance reduction techniques for Monte Carlo simulations of radiative transfer in
// cloudy atmospheres: The solution", JQSRT 112, 434-447.
//
// At a particle scatter, with probability epsilon the new direction is drawn about a
// detector direction (a view picked uniformly) from the particle's own cosine proposal,
// with a uniform azimuth; otherwise the analog polarized sampler runs. Either way the
// weight is multiplied by p_analog / q, q = (1 - epsilon) p_analog + epsilon p_detector,
// so every estimate keeps the analog expectation. p_analog is the density of what the
// analog sampler draws: the bound CDF interpolated linearly in cosine (a density constant
// between table nodes) thinned by the acceptance pdf / bound, normalized by Z.
// Russian roulette after every scatter: a photon lighter than `roulette` survives with
// probability weight / roulette at weight `roulette`.
// ---------------------------------------------------------------------------------
struct Guide {
    double epsilon = 0.0;
    double roulette = 0.0;
    double cap = 1.0e300;         // DDIS only while the weight is below this
    const double* scale = nullptr;  // per-cell roulette threshold scale (nx * ny * nz), or none
    double split = 0.0;           // split above split x the cell's roulette weight (0 = off)
};

// Splitting (the upper bound of a weight window): after an atmospheric scatter, a photon
// heavier than split x W (W = the roulette weight of its cell) continues as n = min(weight /
// W, kSplitMax) copies of weight / n; the copies wait on a stack of kSplitStack per history,
// which also bounds n, and each runs with its own stream (lineage = split_lineage of the
// parent's lineage, its draws so far and the copy's index) once the history before it ends.
constexpr int kSplitMax = 8;
constexpr int kSplitStack = 8;

uint32_t split_lineage(uint32_t lineage, uint32_t draws, uint32_t copy) {
    uint32_t h = lineage * 0x9E3779B1u ^ draws * 0x85EBCA77u ^ copy * 0xC2B2AE3Du;
    h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
    return h ? h : 1u;
}

// Importance tally: for every event, the Stokes-I peel-off contributions of that event and
// of the next kRing - 1 events of the same history, per unit weight at the event, summed
// per cell with the event count. A pilot of the analog method yields the detector
// importance of each cell (mean future contribution of a unit-weight photon there).
constexpr int kRing = 8;

// Density per unit cosine of the analog cosine proposal of species sp.
double proposal_density(const Species& sp, double cs) {
    int hi = int(std::upper_bound(sp.cosines.begin(), sp.cosines.end(), cs) - sp.cosines.begin());
    hi = std::min(std::max(hi, 1), sp.n - 1);
    const int lo = hi - 1;
    return (sp.cdf[size_t(hi)] - sp.cdf[size_t(lo)]) / (sp.cosines[size_t(hi)] - sp.cosines[size_t(lo)]);
}

// Z = integral over the cosine of proposal density x F11 / (F11 + |F12|), the mass the
// acceptance step keeps (the F12 term averages out over the azimuth). Four-point
// Gauss-Legendre per table interval; exactly sum(dCDF) when F12 = 0 or nmat = 1.
double analog_norm(const Species& sp, int nmat) {
    static const double xg[4] = {-0.8611363115940526, -0.3399810435848563, 0.3399810435848563, 0.8611363115940526};
    static const double wg[4] = {0.3478548451374538, 0.6521451548625461, 0.6521451548625461, 0.3478548451374538};
    double z = 0.0;
    for (int lo = 0; lo + 1 < sp.n; ++lo) {
        const double dc = sp.cdf[size_t(lo) + 1] - sp.cdf[size_t(lo)];
        if (dc == 0.0) continue;
        bool ratio_one = nmat == 1 || (sp.f12[size_t(lo)] == 0.0 && sp.f12[size_t(lo) + 1] == 0.0);
        if (ratio_one) { z += dc; continue; }
        double mean = 0.0;
        for (int q = 0; q < 4; ++q) {
            const double t01 = 0.5 * (xg[q] + 1.0);
            const double f11 = sp.f11[size_t(lo)] + t01 * (sp.f11[size_t(lo) + 1] - sp.f11[size_t(lo)]);
            const double f12 = sp.f12[size_t(lo)] + t01 * (sp.f12[size_t(lo) + 1] - sp.f12[size_t(lo)]);
            const double b = f11 + std::fabs(f12);
            mean += 0.5 * wg[q] * (b > 0.0 ? f11 / b : 0.0);
        }
        z += dc * mean;
    }
    return z;
}

// Cosine drawn from the bound CDF (the proposal step of mie_scatter_pol_bound).
double sample_proposal(const Species& sp, double u) {
    int hi = int(std::upper_bound(sp.cdf.begin(), sp.cdf.end(), u) - sp.cdf.begin());
    hi = std::min(std::max(hi, 1), sp.n - 1);
    const int lo = hi - 1;
    const double c2[2] = {sp.cdf[size_t(lo)], sp.cdf[size_t(hi)]};
    const double a2[2] = {sp.cosines[size_t(lo)], sp.cosines[size_t(hi)]};
    return linpol2(c2, a2, u);
}

// ---------------------------------------------------------------------------------
// Per-round tallies in the RawTallies order: stokes(nmat,nx,ny,angles),
// paths(nx,ny,nz,angles), weights(nx,ny,angles), all Fortran order, FP64.
// ---------------------------------------------------------------------------------
struct Counters {
    uint64_t scatters = 0, photons = 0, free_path_visits = 0, detector_visits = 0, tally_updates = 0;
    void add(const Counters& o) {
        scatters += o.scatters; photons += o.photons; free_path_visits += o.free_path_visits;
        detector_visits += o.detector_visits; tally_updates += o.tally_updates;
    }
};

// Backward transport registers every view at the injection column (reg_i, reg_j) and
// attributes the event to the location of the history's first event (loc_*); forward
// transport projects each view ray to the top (reg_i = 0) and uses the event's own cell.
struct Register { int reg_i = 0, reg_j = 0, loc_i = 0, loc_j = 0, loc_layer = -1; };

struct Transport {
    const Tables& t;
    uint32_t max_steps;
    Guide guide;
    std::vector<double> z_norm;  // analog sampler mass per particle species
    const double* pixel_weight = nullptr;  // importance-tally weight per output pixel, or none
    bool orders = false;     // scattering-order diagnostics (calc_radiances_and_scats)
    size_t orders_offset = 0, locations = 0;
    double a0, b0, c0, phi0_rad, vartheta0_rad;
    std::vector<double> va, vb, vc, view_phi_rad, zsum;  // zsum[k] = SUM(zunit(1:k))
    size_t stokes_count, path_count, weight_count, tally_count;

    Transport(const Tables& tables, uint32_t steps) : t(tables), max_steps(steps) {
        vartheta0_rad = kDegToRad * t.vartheta0;
        phi0_rad = kDegToRad * t.phi0;
        a0 = std::sin(vartheta0_rad) * std::cos(phi0_rad);
        b0 = std::sin(vartheta0_rad) * std::sin(phi0_rad);
        c0 = std::cos(vartheta0_rad);
        for (int ia = 0; ia < t.angles; ++ia) {
            double th = kDegToRad * t.vartheta[ia], ph = kDegToRad * t.view_phi[ia];
            va.push_back(std::cos(ph) * std::sin(th));
            vb.push_back(std::sin(ph) * std::sin(th));
            vc.push_back(std::cos(th));
            view_phi_rad.push_back(ph);
        }
        zsum.assign(t.nz + 1, 0.0);
        for (int k = 1; k <= t.nz; ++k) zsum[k] = zsum[k - 1] + t.zu(k);
        stokes_count = size_t(t.nmat) * t.nx * t.ny * t.angles;
        path_count = t.paths ? size_t(t.nx) * t.ny * t.nz * t.angles : 0;
        weight_count = t.paths ? size_t(t.nx) * t.ny * t.angles : 0;
        tally_count = stokes_count + path_count + weight_count;
        for (const auto& sp : t.species) z_norm.push_back(analog_norm(sp, t.nmat));
    }

    // Scattering-order diagnostics after the weights: single-scattering Stokes, then the
    // contribution per event location (nmat, nx, ny, 0:nz-1, angles; layer 0 = surface) of
    // all orders and of single scattering (mc_routines_cartesian_mod.f90:405-836).
    void enable_orders() {
        orders = true;
        orders_offset = tally_count;
        locations = size_t(t.nx) * t.ny * t.nz * t.angles;
        tally_count += stokes_count + 2 * size_t(t.nmat) * locations;
    }
    size_t location_index(int m, int i, int j, int layer, int ia) const {
        return size_t(m) + size_t(t.nmat) * (size_t(i - 1) + size_t(t.nx) * (size_t(j - 1) + size_t(t.ny) * (size_t(layer) + size_t(t.nz) * size_t(ia))));
    }

    // Russian roulette; false when the photon is terminated.
    bool roulette(double& weight, Stream& rng, int i, int j, int k) const {
        double threshold = guide.roulette;
        if (guide.scale) threshold *= guide.scale[size_t(i - 1) + size_t(t.nx) * (size_t(j - 1) + size_t(t.ny) * size_t(k - 1))];
        if (!(threshold > 0.0) || !(weight < threshold)) return true;
        if (rng.uniform() * threshold < weight) { weight = threshold; return true; }
        return false;
    }

    // DDIS weight factor p_analog / q for a particle scatter into (a, b, c) at cos_sca;
    // s0 is the scattered intensity (the acceptance pdf) for the unit incident Stokes vector.
    double ddis_factor(int sp_index, double cos_sca, double s0, double a, double b, double c) const {
        const Species& sp = t.species[size_t(sp_index)];
        double f11, f12;
        mie_scat_elements(cos_sca, sp, f11, f12);
        if (t.nmat == 1) f12 = 0.0;
        const double bound = f11 + std::fabs(f12);
        const double p_an = bound > 0.0 ? proposal_density(sp, cos_sca) * (s0 / bound) / z_norm[size_t(sp_index)] : 0.0;
        double p_det = 0.0;
        for (int v = 0; v < t.angles; ++v) {
            double cv = a * va[size_t(v)] + b * vb[size_t(v)] + c * vc[size_t(v)];
            p_det += proposal_density(sp, std::min(1.0, std::max(-1.0, cv)));
        }
        p_det /= double(t.angles);
        const double q = (1.0 - guide.epsilon) * p_an + guide.epsilon * p_det;
        return q > 0.0 ? p_an / q : 0.0;
    }

    size_t stokes_index(int m, int i, int j, int ia) const {
        return size_t(m) + size_t(t.nmat) * (size_t(i - 1) + size_t(t.nx) * (size_t(j - 1) + size_t(t.ny) * size_t(ia)));
    }
    size_t path_index(int i, int j, int k, int ia) const {
        return stokes_count + size_t(i - 1) + size_t(t.nx) * (size_t(j - 1) + size_t(t.ny) * (size_t(k - 1) + size_t(t.nz) * size_t(ia)));
    }
    size_t weight_index(int i, int j, int ia) const {
        return stokes_count + path_count + size_t(i - 1) + size_t(t.nx) * (size_t(j - 1) + size_t(t.ny) * size_t(ia));
    }

    // ADVANCE / ADVANCE_internal (identical bodies; mc.f90:1531-1580).
    void advance(int& i, int& j, int& k, double& x, double& y, double& z, int is, int js, int ks,
                 double aa, double ba, double ca, double ai, double bi, double ci, double& dist) const {
        double dx = x * ai, dy = y * bi, dz = z * ci;
        dist = std::min(dx, std::min(dy, dz));
        if (dx == dist) {
            i = (i + is + t.nx - 1) % t.nx + 1;
            x = t.xunit;
            y = std::max(0.0, y - ba * dist);
            z = std::max(0.0, z - ca * dist);
        } else if (dy == dist) {
            j = (j + js + t.ny - 1) % t.ny + 1;
            x = std::max(0.0, x - aa * dist);
            y = t.yunit;
            z = std::max(0.0, z - ca * dist);
        } else {
            k = k + ks;
            x = std::max(0.0, x - aa * dist);
            y = std::max(0.0, y - ba * dist);
            if (k >= 1 && k <= t.nz) z = t.zu(k);
        }
    }

    // calc_radiances_pol / calc_radiances_and_paths_pol (mc_routines_cartesian_mod.f90).
    // Returns false when a detector ray exceeds the step cap.
    bool peel_off(double a_bak, double b_bak, double c_bak, int i_bak, int j_bak, int k_bak,
                  double x_bak, double y_bak, double z_bak, const std::vector<double>& s_prob,
                  const std::vector<double>& path_layers, double* tally,
                  std::vector<double>& path_angle, Counters& cnt, double& contributed,
                  uint32_t nscat = 0, const Register& reg = Register()) const {
        const int nmat = t.nmat, nz = t.nz;
        contributed = 0.0;
        for (int ia = 0; ia < t.angles; ++ia) {
            double p1 = s_prob[size_t(ia) * nmat];
            if (!(p1 > kEps)) continue;
            double a = va[ia], b = vb[ia], c = vc[ia];
            int i = i_bak, j = j_bak, k = k_bak;
            double x = x_bak, y = y_bak, z = z_bak;
            if (a * a_bak < 0.0) x = std::max(0.0, t.xunit - x);
            if (b * b_bak < 0.0) y = std::max(0.0, t.yunit - y);
            if (c * c_bak < 0.0) z = std::max(0.0, t.zu(k) - z);
            double tau = 0.0;
            if (t.paths) std::fill(path_angle.begin(), path_angle.end(), 0.0);
            int is = int(fortran_sign(1.0, a)), js = int(fortran_sign(1.0, b)), ks = int(fortran_sign(1.0, c));
            double aa = std::fabs(a), ba = std::fabs(b), ca = std::fabs(c);
            double ai = 1.0 / std::max(aa, kEps), bi = 1.0 / std::max(ba, kEps), ci = 1.0 / std::max(ca, kEps);
            double x_old = x, y_old = y, z_old = z;
            uint32_t steps = 0;
            while (k >= 1 && k < nz) {
                if (++steps > max_steps) return false;
                double bv = t.beta_at(i, j, k);
                int k_old = k;
                double dist;
                advance(i, j, k, x, y, z, is, js, ks, aa, ba, ca, ai, bi, ci, dist);
                tau += dist * bv;
                if (t.paths) path_angle[size_t(k_old - 1)] += dist;
                ++cnt.detector_visits;
            }
            // Register grid mapping (k_register == k_detector == nz: direction = +1).
            double height = zsum[size_t(k_bak - 1)];
            height += ks > 0 ? t.zu(k_bak) - z_old : z_old;
            height = zsum[size_t(nz - 1)] - height;
            double delta_x = aa * height / ca, delta_y = ba * height / ca;
            int di = int(((t.xunit - x_old) + delta_x) / t.xunit);
            int dj = int(((t.yunit - y_old) + delta_y) / t.yunit);
            auto modulo = [](long long v, long long m) { long long r = v % m; return r < 0 ? r + m : r; };
            int inew = int(modulo((long long)i_bak + is * (long long)di + t.nx - 1, t.nx)) + 1;
            int jnew = int(modulo((long long)j_bak + js * (long long)dj + t.ny - 1, t.ny)) + 1;
            if (reg.reg_i > 0) { inew = reg.reg_i; jnew = reg.reg_j; }
            double att = std::exp(-tau);
            contributed += pixel_weight ? p1 * att * pixel_weight[size_t(inew - 1) + size_t(t.nx) * (size_t(jnew - 1) + size_t(t.ny) * size_t(ia))]
                                        : p1 * att;
            for (int m = 0; m < nmat; ++m) tally[stokes_index(m, inew, jnew, ia)] += s_prob[size_t(ia) * nmat + m] * att;
            cnt.tally_updates += nmat;
            if (orders) {
                int li = i_bak, lj = j_bak, layer = (k_bak == 1 && z_bak < kEps) ? 0 : k_bak;
                if (reg.loc_layer >= 0) { li = reg.loc_i; lj = reg.loc_j; layer = reg.loc_layer; }
                for (int m = 0; m < nmat; ++m) {
                    const double v = s_prob[size_t(ia) * nmat + m] * att;
                    tally[orders_offset + stokes_count + location_index(m, li, lj, layer, ia)] += v;
                    if (nscat == 1) {
                        tally[orders_offset + stokes_index(m, inew, jnew, ia)] += v;
                        tally[orders_offset + stokes_count + size_t(nmat) * locations + location_index(m, li, lj, layer, ia)] += v;
                    }
                }
            }
            if (t.paths) {
                double c1 = p1 * att;
                for (int kk = 1; kk <= nz; ++kk)
                    tally[path_index(inew, jnew, kk, ia)] += c1 * (path_layers[size_t(kk - 1)] + path_angle[size_t(kk - 1)]);
                tally[weight_index(inew, jnew, ia)] += c1;
                cnt.tally_updates += nz + 1;
            }
        }
        return true;
    }

    // One photon history (mc.f90:351-1436). Returns a failure flag (0 on success).
    uint32_t photon(uint32_t photon_id, uint32_t round, uint32_t seed, double* tally,
                    Counters& cnt, std::vector<double>& path_layers, std::vector<double>& path_angle,
                    std::vector<double>& s_prob, double* importance) const {
        const int nx = t.nx, ny = t.ny, nz = t.nz, nmat = t.nmat;
        uint32_t ring_cell[kRing];
        double ring_inv[kRing];
        int ring_n = 0;
        double contributed = 0.0;
        uint32_t nscat = 0;  // events of this history so far (its scattering order)
        // Record an event in cell (i, j, k) at weight w that contributed c.
        auto record = [&](int ci, int cj, int ck, double w, double c) {
            if (!importance) return;
            const size_t cells = size_t(nx) * ny * nz;
            const uint32_t cell = uint32_t(size_t(ci - 1) + size_t(nx) * (size_t(cj - 1) + size_t(ny) * size_t(ck - 1)));
            ring_cell[ring_n % kRing] = cell;
            ring_inv[ring_n % kRing] = 1.0 / w;
            ++ring_n;
            importance[cells + cell] += 1.0;
            const int live = std::min(ring_n, kRing);
            for (int e = 0; e < live; ++e) importance[ring_cell[e]] += c * ring_inv[e];
        };
        Stream rng{photon_id, round, seed};
        ++cnt.photons;
        int column = int(photon_id % uint32_t(nx * ny));
        int i = column % nx + 1;
        int j = std::min(column / nx + 1, ny);
        int k = t.k_source;
        double x = t.xunit * rng.uniform();
        double y = t.yunit * rng.uniform();
        double z = t.zu(k);
        double s[4] = {1.0, 0.0, 0.0, 0.0};
        double weight = 1.0;
        // Backward transport: the weight matrix (identity at injection), the injection
        // column where every contribution registers, and the first event's location.
        const bool backward = t.backward;
        const double sign = backward ? 1.0 : -1.0;
        double M[4][4] = {};
        for (int m = 0; m < nmat; ++m) M[m][m] = 1.0;
        Register reg;
        if (backward) { reg.reg_i = i; reg.reg_j = j; }
        auto locate = [&](int ei, int ej, int ek, double ez) {
            if (!backward) return;
            if (nscat == 1) { reg.loc_i = ei; reg.loc_j = ej; reg.loc_layer = (ek == 1 && ez < kEps) ? 0 : ek; }
        };
        if (t.paths) std::fill(path_layers.begin(), path_layers.end(), 0.0);
        double a = a0, b = b0, c = c0, phi_in = phi0_rad;
        double remains = 0;
        bool new_path = true;  // label 1000 (draw a new optical path) vs 1010
        uint32_t steps = 0;
        // Copies made by splitting, run after the history before them ends (last first).
        struct Copy {
            int i, j, k;
            double x, y, z, a, b, c, phi, s[4], weight;
            uint32_t steps, nscat, lineage;
        };
        Copy pending[kSplitStack];
        int waiting = 0;
    history:
        for (;;) {
            if (new_path) remains = -std::log(std::max(rng.uniform(), kEps));
            new_path = false;
            // label 1010
            int is = int(fortran_sign(1.0, a)), js = int(fortran_sign(1.0, b)), ks = int(fortran_sign(1.0, c));
            double aa = std::fabs(a), ba = std::fabs(b), ca = std::fabs(c);
            double ai = 1.0 / std::max(aa, kEps), bi = 1.0 / std::max(ba, kEps), ci = 1.0 / std::max(ca, kEps);
            bool surface = false, event = false;
            // label 1020 loop
            for (;;) {
                if (++steps > max_steps) return 16;
                ++cnt.free_path_visits;
                double bv = (k < nz && k > 0) ? t.beta_at(i, j, k) : 0.0;
                if (bv > kEps) {
                    double de = remains / bv;
                    if (de < x * ai && de < y * bi && de < z * ci) {
                        x = std::max(0.0, x - aa * de);
                        y = std::max(0.0, y - ba * de);
                        z = std::max(0.0, z - ca * de);
                        if (t.paths) path_layers[size_t(k - 1)] += de;
                        event = true;
                        break;
                    }
                }
                int k_old = k;
                double dist;
                advance(i, j, k, x, y, z, is, js, ks, aa, ba, ca, ai, bi, ci, dist);
                if (t.paths) path_layers[size_t(k_old - 1)] += dist;
                remains -= dist * bv;
                if (k <= nz && k >= 1) continue;
                if (k > nz) goto ended;  // escaped through TOA
                surface = true;
                break;
            }
            if (surface) {
                double a_int = a, b_int = b, c_int = c;
                k = std::max(k, 1);
                z = 0.0;
                weight *= t.albedo[size_t(i - 1) + size_t(nx) * size_t(j - 1)];
                if (weight < kEps) goto ended;
                ++cnt.scatters;
                ++nscat;
                locate(i, j, k, z);
                for (int ia = 0; ia < t.angles; ++ia) {
                    for (int m = 0; m < nmat; ++m) s_prob[size_t(ia) * nmat + m] = 0.0;
                    if (vc[ia] > 0) {
                        // Forward As S (only I survives); backward M As S0 (the first column of M).
                        if (backward) for (int m = 0; m < nmat; ++m) s_prob[size_t(ia) * nmat + m] = M[m][0] * vc[ia] * weight;
                        else s_prob[size_t(ia) * nmat] = s[0] * vc[ia] * weight;
                    }
                    for (int m = 0; m < (backward ? nmat : 1); ++m)
                        if (!std::isfinite(s_prob[size_t(ia) * nmat + m])) return 1;
                }
                if (!peel_off(a_int, b_int, c_int, i, j, k, x, y, z, s_prob, path_layers, tally, path_angle, cnt, contributed,
                              nscat, reg))
                    return 2;
                record(i, j, k, weight, contributed);
                // GROUND_LAMB2: theta = acos(sqrt(P)), phi = 2 pi U.
                double P = rng.uniform(), U = rng.uniform();
                if (!roulette(weight, rng, i, j, k)) goto ended;
                double theta = std::acos(std::sqrt(P));
                double phi_out = 2.0 * kPi * U;
                a = std::sin(theta) * std::cos(phi_out);
                b = std::sin(theta) * std::sin(phi_out);
                c = std::fabs(std::cos(theta));
                if (backward) {
                    // M As keeps the first column; the sampling vector is (M11, 0, 0, 0).
                    for (int r = 0; r < nmat; ++r) for (int col = 1; col < nmat; ++col) M[r][col] = 0.0;
                    s[0] = M[0][0];
                }
                s[1] = 0.0; s[2] = 0.0; s[3] = 0.0;  // As * S keeps only I
                if (s[0] > kEps) { double s0 = s[0]; for (int m = 0; m < nmat; ++m) s[m] /= s0; }
                if (backward) {
                    const double m11 = M[0][0];
                    for (int r = 0; r < nmat; ++r) for (int col = 0; col < nmat; ++col) M[r][col] /= m11;
                }
                if (a * a_int < 0.0) x = std::max(0.0, t.xunit - x);
                if (b * b_int < 0.0) y = std::max(0.0, t.yunit - y);
                if (c * c_int < 0.0) z = std::max(0.0, t.zu(k) - z);
                phi_in = phi_out;
                continue;  // GOTO 1010 (keeps remains)
            }
            (void)event;
            // label 3000: species selection (gas is index ntypes + 1).
            double rtemp = rng.uniform();
            int sp = 1;
            double work = t.fraction_at(1, i, j, k);
            while (work <= rtemp && sp < t.ntypes + 1) {
                ++sp;
                work += t.fraction_at(sp, i, j, k);
            }
            bool gas = sp == t.ntypes + 1;
            weight *= gas ? t.ssalb_gas[size_t(k - 1)] : t.species[size_t(sp - 1)].ssalb;
            if (weight < kEps) goto ended;
            ++cnt.scatters;
            ++nscat;
            locate(i, j, k, z);
            for (int ia = 0; ia < t.angles; ++ia) {
                double cs = c * vc[ia] + std::sqrt(std::max(kEps, 1.0 - c * c)) *
                                             std::sqrt(std::max(kEps, 1.0 - vc[ia] * vc[ia])) *
                                             std::cos(phi_in - view_phi_rad[ia]);
                Rotation rot = stokes_rot_mat(cs, c, vc[ia], phi_in, view_phi_rad[ia], nmat);
                Mat4 f = gas ? ray_scat_matrix(nmat, cs, t.depol) : mie_scat_matrix(nmat, cs, t.species[size_t(sp - 1)]);
                Mat4 p = matmul_stokes_rot(nmat, f, rot);
                double back[4];
                if (backward) {
                    // M P^T S0: M times the first row of P.
                    for (int r = 0; r < nmat; ++r) {
                        double acc = 0.0;
                        for (int col = 0; col < nmat; ++col) acc += M[r][col] * p.m[0][col];
                        back[r] = acc;
                    }
                } else {
                    apply(nmat, p, s, back);
                }
                for (int m = 0; m < nmat; ++m) s_prob[size_t(ia) * nmat + m] = back[m] * weight;
                if (s_prob[size_t(ia) * nmat] < 1.0e-100)
                    for (int m = 0; m < nmat; ++m) s_prob[size_t(ia) * nmat + m] = 0.0;
                for (int m = 0; m < nmat; ++m)
                    if (!std::isfinite(s_prob[size_t(ia) * nmat + m])) return 1;
            }
            if (!peel_off(a, b, c, i, j, k, x, y, z, s_prob, path_layers, tally, path_angle, cnt, contributed, nscat, reg))
                return 2;
            record(i, j, k, weight, contributed);
            double cos_in = c, cos_out, dphi, cos_sca, phi_out;
            const bool guided = !gas && guide.epsilon > 0.0 && weight < guide.cap;
            if (guided && rng.uniform() < guide.epsilon) {
                // Detector branch: a view, a cosine about it from the proposal, an azimuth.
                const int v = std::min(int(rng.uniform() * t.angles), t.angles - 1);
                const double cd = sample_proposal(t.species[size_t(sp - 1)], rng.uniform());
                const double psi = 2.0 * kPi * rng.uniform();
                const double dx = va[size_t(v)], dy = vb[size_t(v)], dz = vc[size_t(v)];
                const double h = std::sqrt(dx * dx + dy * dy);
                const double e1x = h > 1e-12 ? -dy / h : 1.0, e1y = h > 1e-12 ? dx / h : 0.0;
                const double e2x = -dz * e1y, e2y = dz * e1x, e2z = dx * e1y - dy * e1x;
                const double sd = std::sqrt(std::max(0.0, 1.0 - cd * cd));
                const double cp = std::cos(psi), spsi = std::sin(psi);
                const double wx = cd * dx + sd * (cp * e1x + spsi * e2x);
                const double wy = cd * dy + sd * (cp * e1y + spsi * e2y);
                const double wz = cd * dz + sd * spsi * e2z;
                cos_out = std::min(1.0, std::max(-1.0, wz));
                phi_out = std::atan2(wy, wx);
                const double so = std::sqrt(std::max(0.0, 1.0 - cos_out * cos_out));
                cos_sca = std::min(1.0, std::max(-1.0, a * (std::cos(phi_out) * so) + b * (std::sin(phi_out) * so) + c * cos_out));
            } else {
                bool ok = gas ? rayl_scatter_pol(nmat, t.depol, s, cos_in, rng, cos_out, dphi, cos_sca, sign)
                              : mie_scatter_pol_bound(nmat, t.species[size_t(sp - 1)], s, cos_in, rng, cos_out, dphi, cos_sca, sign);
                if (!ok) return 4;
                phi_out = phi_in + dphi;
            }
            Rotation rot = stokes_rot_mat(cos_sca, cos_in, cos_out, phi_in, phi_out, nmat);
            Mat4 f = gas ? ray_scat_matrix(nmat, cos_sca, t.depol) : mie_scat_matrix(nmat, cos_sca, t.species[size_t(sp - 1)]);
            Mat4 p = matmul_stokes_rot(nmat, f, rot);
            double ns[4];
            if (backward) {
                // M = M P^T; the sampling vector is (M11, M12, -M13, M14).
                double next[4][4] = {};
                for (int r = 0; r < nmat; ++r)
                    for (int col = 0; col < nmat; ++col) {
                        double acc = 0.0;
                        for (int q = 0; q < nmat; ++q) acc += M[r][q] * p.m[col][q];
                        next[r][col] = acc;
                    }
                std::memcpy(M, next, sizeof(M));
                ns[0] = M[0][0];
                if (nmat > 1) { ns[1] = M[0][1]; ns[2] = -M[0][2]; }
                if (nmat > 3) ns[3] = M[0][3];
            } else {
                apply(nmat, p, s, ns);
            }
            double s0 = ns[0];
            for (int m = 0; m < nmat; ++m) s[m] = ns[m] / s0;
            if (s[0] < 1.0e-100) for (int m = 0; m < nmat; ++m) s[m] = 0.0;
            for (int m = 0; m < nmat; ++m) if (!std::isfinite(s[m])) return 8;
            if (nmat == 3 && std::sqrt(s[1] * s[1] + s[2] * s[2]) > s[0] + kStokesCriterium) return 8;
            if (nmat == 4 && std::sqrt(s[1] * s[1] + s[2] * s[2] + s[3] * s[3]) > s[0] + kStokesCriterium) return 8;
            if (backward) {
                const double m11 = M[0][0];
                for (int r = 0; r < nmat; ++r) for (int col = 0; col < nmat; ++col) M[r][col] /= m11;
            }
            double a_bak = a, b_bak = b, c_bak = c;
            a = std::cos(phi_out) * std::sqrt(std::max(0.0, 1.0 - cos_out * cos_out));
            b = std::sin(phi_out) * std::sqrt(std::max(0.0, 1.0 - cos_out * cos_out));
            c = cos_out;
            if (guided) weight *= ddis_factor(sp - 1, cos_sca, s0, a, b, c);
            if (!roulette(weight, rng, i, j, k)) goto ended;
            if (a * a_bak < 0.0) x = std::max(0.0, t.xunit - x);
            if (b * b_bak < 0.0) y = std::max(0.0, t.yunit - y);
            if (c * c_bak < 0.0) z = std::max(0.0, t.zu(k) - z);
            phi_in = phi_out;
            if (guide.split > 0.0) {
                double w_cell = guide.roulette;
                if (guide.scale) w_cell *= guide.scale[size_t(i - 1) + size_t(nx) * (size_t(j - 1) + size_t(ny) * size_t(k - 1))];
                if (w_cell > 0.0 && weight > guide.split * w_cell) {
                    const int n = std::min({int(weight / w_cell), kSplitMax, 1 + kSplitStack - waiting});
                    if (n >= 2) {
                        weight /= double(n);
                        for (int copy = 1; copy < n; ++copy) {
                            Copy& p = pending[waiting++];
                            p = Copy{i, j, k, x, y, z, a, b, c, phi_in, {s[0], s[1], s[2], s[3]}, weight, steps, nscat,
                                     split_lineage(rng.lineage, rng.draws, uint32_t(copy))};
                        }
                    }
                }
            }
            new_path = true;  // GOTO 1000
        }
    ended:
        // The history ended (GOTO 4000); a copy left by splitting continues the photon.
        if (waiting > 0) {
            const Copy& p = pending[--waiting];
            i = p.i; j = p.j; k = p.k; x = p.x; y = p.y; z = p.z; a = p.a; b = p.b; c = p.c; phi_in = p.phi;
            for (int m = 0; m < 4; ++m) s[m] = p.s[m];
            weight = p.weight; steps = p.steps; nscat = p.nscat;
            rng = Stream{photon_id, round, seed, p.lineage};
            new_path = true;
            goto history;
        }
        return 0;
    }
};

void write_error(char* err, size_t n, const std::string& msg) {
    if (err && n) std::snprintf(err, n, "%s", msg.c_str());
}

}  // namespace

extern "C" {

int monki_oracle_abi_version(void) { return 1; }

// Philox4x32-10 of one counter/key pair (known-answer tests).
void monki_oracle_philox(const uint32_t counter[4], const uint32_t key[2], uint32_t out[4]) {
    uint32_t ctr[4] = {counter[0], counter[1], counter[2], counter[3]};
    philox(ctr, key);
    std::memcpy(out, ctr, sizeof(ctr));
}

// One uniform draw sequence of a photon stream: n values of Stream::uniform().
void monki_oracle_uniforms(uint32_t photon, uint32_t round, uint32_t seed, uint32_t n, double* out) {
    Stream s{photon, round, seed};
    for (uint32_t i = 0; i < n; ++i) out[i] = s.uniform();
}

// The polarization probe: ray_scat_matrix, stokes_rot_mat and matmul_stokes_rot applied
// to S (tests/native/metal_probe.f90 of the reference).
void monki_oracle_scatter_stokes(double depol, double uo, double u1, double phio, double phi1,
                                 const double stokes[3], double out[3]) {
    double cs = uo * u1 + std::sqrt(1 - uo * uo) * std::sqrt(1 - u1 * u1) * std::cos(phio - phi1);
    Mat4 f = ray_scat_matrix(3, cs, depol);
    Rotation r = stokes_rot_mat(cs, uo, u1, phio, phi1, 3);
    Mat4 p = matmul_stokes_rot(3, f, r);
    apply(3, p, stokes, out);
}

// Validate a transport table stream; 0 on success, else the message in err.
int monki_oracle_validate(const double* tables, size_t count, char* err, size_t errlen) {
    try {
        parse_tables(tables, count);
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

// Run photons [first, first + count) of the flattened round group, exactly like one
// monki_cuda_run call. controls: count, first photon, first round, seed, max_steps,
// profile (ignored), photons per round, active rounds. out: active rounds x tally
// count FP64, each round in RawTallies order with the mu0/mu factor applied to Stokes.
// counters (5 x u64): scatters, photons, free-path cell visits, detector cell visits,
// tally updates. Returns the failure flag (0 on success); a nonzero flag rejects the run.
int monki_oracle_run_guided(const double* tables, size_t table_count, const uint32_t controls[8],
                            const double guide[4], const double* scale, int threads, double* out,
                            uint64_t* counters, double* importance, const double* pixel_weight,
                            uint32_t options, char* err, size_t errlen);

int monki_oracle_run(const double* tables, size_t table_count, const uint32_t controls[8], int threads,
                     double* out, uint64_t* counters, char* err, size_t errlen) {
    const double plain[4] = {0.0, 0.0, 0.0, 0.0};
    return monki_oracle_run_guided(tables, table_count, controls, plain, nullptr, threads, out, counters, nullptr,
                                   nullptr, 0u, err, errlen);
}

// The same round group with guided transport: guide = {epsilon (DDIS probability at
// particle scatters, [0, 1)), roulette weight (0 = off), DDIS weight cap (0 = none),
// splitting factor (0 = off, else >= 1: split above that many roulette weights)};
// scale (nx * ny * nz, or NULL) multiplies the roulette weight per cell. importance
// (2 * nx * ny * nz, or NULL) receives the importance tally: per cell the summed future
// contribution per unit weight, then the event count; pixel_weight (nx * ny * angles, or
// NULL) weights each contribution by its output pixel. options bit 0 adds the
// scattering-order diagnostics to each round's tallies.
int monki_oracle_run_guided(const double* tables, size_t table_count, const uint32_t controls[8],
                            const double guide[4], const double* scale, int threads, double* out,
                            uint64_t* counters, double* importance, const double* pixel_weight,
                            uint32_t options, char* err, size_t errlen) {
    try {
        if (!guide || !(guide[0] >= 0.0 && guide[0] < 1.0) || !(guide[1] >= 0.0 && guide[1] <= 1.0)) {
            write_error(err, errlen, "Invalid guide: epsilon must be in [0, 1), roulette in [0, 1]");
            return 1;
        }
        Tables t = parse_tables(tables, table_count);
        const uint32_t count = controls[0], first = controls[1], first_round = controls[2];
        const uint32_t seed = controls[3], max_steps = controls[4], per_round = controls[6];
        const uint32_t rounds = controls[7];
        if (!per_round || !rounds || uint64_t(first) + count > uint64_t(per_round) * rounds) {
            write_error(err, errlen, "Invalid round group");
            return 1;
        }
        if (!(guide[3] == 0.0 || (guide[3] >= 1.0 && std::isfinite(guide[3])))) {
            write_error(err, errlen, "Invalid guide: split must be 0 or at least 1");
            return 1;
        }
        if (guide[3] > 0.0 && (t.paths || importance || guide[1] <= 0.0)) {
            write_error(err, errlen, "Splitting needs a roulette weight and no layer paths or importance tallies");
            return 1;
        }
        if (t.backward && (guide[0] > 0.0 || guide[1] > 0.0 || importance || pixel_weight)) {
            write_error(err, errlen, "Guided transport and importance tallies need forward transport");
            return 1;
        }
        Transport tr(t, max_steps);
        tr.guide.epsilon = guide[0];
        tr.guide.roulette = guide[1];
        if (guide[2] > 0.0) tr.guide.cap = guide[2];
        tr.guide.split = guide[3];
        tr.guide.scale = scale;
        tr.pixel_weight = pixel_weight;
        if (options & 1u) tr.enable_orders();
        const size_t cells = size_t(t.nx) * t.ny * t.nz;
        if (scale)
            for (size_t c = 0; c < cells; ++c)
                if (!(scale[c] >= 0.0) || !std::isfinite(scale[c])) {
                    write_error(err, errlen, "Invalid roulette scale map");
                    return 1;
                }
        std::vector<std::vector<double>> imp_partial(importance ? size_t(threads > 0 ? threads : 1) : 0,
                                                     std::vector<double>(importance ? 2 * cells : 0, 0.0));
        const size_t tc = tr.tally_count;
        std::fill(out, out + tc * rounds, 0.0);
        int nthreads = threads > 0 ? threads : 1;
        std::vector<std::vector<double>> partial(size_t(nthreads), std::vector<double>(tc * rounds, 0.0));
        std::vector<Counters> cnts(static_cast<size_t>(nthreads));
        std::vector<uint32_t> flags(static_cast<size_t>(nthreads), 0u);
        std::vector<std::string> errors(static_cast<size_t>(nthreads));
#pragma omp parallel num_threads(nthreads)
        {
            int tid = 0;
#ifdef _OPENMP
            tid = omp_get_thread_num();
#endif
            std::vector<double> path_layers(size_t(t.nz), 0.0), path_angle(size_t(t.nz), 0.0);
            std::vector<double> s_prob(size_t(t.angles) * t.nmat, 0.0);
#pragma omp for schedule(dynamic, 256)
            for (long long n = 0; n < (long long)count; ++n) {
                if (flags[size_t(tid)]) continue;
                uint32_t identity = first + uint32_t(n);
                uint32_t round_offset = identity / per_round;
                uint32_t photon_id = identity % per_round;
                double* tally = partial[size_t(tid)].data() + size_t(round_offset) * tc;
                try {
                    uint32_t flag = tr.photon(photon_id, first_round + round_offset, seed, tally,
                                              cnts[size_t(tid)], path_layers, path_angle, s_prob,
                                              importance ? imp_partial[size_t(tid)].data() : nullptr);
                    if (flag) flags[size_t(tid)] |= flag;
                } catch (const std::exception& e) {
                    errors[size_t(tid)] = e.what();
                    flags[size_t(tid)] |= 0x100;
                }
            }
        }
        uint32_t flag = 0;
        Counters total;
        for (int q = 0; q < nthreads; ++q) {
            flag |= flags[size_t(q)];
            total.add(cnts[size_t(q)]);
            const std::vector<double>& p = partial[size_t(q)];
            for (size_t v = 0; v < tc * rounds; ++v) out[v] += p[v];
            if (importance) {
                if (q == 0) std::fill(importance, importance + 2 * cells, 0.0);
                for (size_t v = 0; v < 2 * cells; ++v) importance[v] += imp_partial[size_t(q)][v];
            }
        }
        // mu0/mu geometry factor on Stokes only, forward transport only (mc.f90:1456-1474).
        for (uint32_t r = 0; r < (t.backward ? 0u : rounds); ++r)
            for (int ia = 0; ia < t.angles; ++ia) {
                double f = std::fabs(std::cos(tr.vartheta0_rad)) / std::fabs(std::cos(kDegToRad * t.vartheta[ia]));
                for (int j = 1; j <= t.ny; ++j)
                    for (int i = 1; i <= t.nx; ++i)
                        for (int m = 0; m < t.nmat; ++m) {
                            out[size_t(r) * tc + tr.stokes_index(m, i, j, ia)] *= f;
                            if (tr.orders) {
                                out[size_t(r) * tc + tr.orders_offset + tr.stokes_index(m, i, j, ia)] *= f;
                                for (int layer = 0; layer < t.nz; ++layer) {
                                    const size_t at = size_t(r) * tc + tr.orders_offset + tr.stokes_count + tr.location_index(m, i, j, layer, ia);
                                    out[at] *= f;
                                    out[at + size_t(t.nmat) * tr.locations] *= f;
                                }
                            }
                        }
            }
        if (counters) {
            counters[0] = total.scatters; counters[1] = total.photons; counters[2] = total.free_path_visits;
            counters[3] = total.detector_visits; counters[4] = total.tally_updates;
        }
        if (flag) {
            std::string msg;
            for (const auto& e : errors) if (!e.empty()) { msg = e; break; }
            if (msg.empty()) msg = "Oracle transport failed (flag " + std::to_string(flag) + "); round rejected";
            write_error(err, errlen, msg);
            return int(flag);
        }
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 0x100;
    }
}

}  // extern "C"
