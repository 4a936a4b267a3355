// Device physics of one photon history: Philox streams, scattering matrices, Stokes
// rotation and polarized direction sampling. Templated on the transport scalar T:
// float is the product path; double is the FP64 transport build that states the FP32
// bias. Both follow the same formulas; only the degeneracy tolerances are scaled to T.
//
// Reference formulas (paths relative to the reference project):
//   Philox stream layout      kernels/metal/transport.metal:64-92
//   ray_scat_matrix           fortran/.../modules/mc_routines_general_mod.f90:74-136
//   mie_scat_matrix           fortran/.../modules/mc_routines_general_mod.f90:257-388
//   rayl_scatter_pol          fortran/.../modules/mc_routines_general_mod.f90:492-670
//   mie_scatter_pol_bound     fortran/.../modules/mc_routines_general_mod.f90:682-932
//   stokes_rot_mat            fortran/.../modules/mc_routines_general_mod.f90:942-1174
//   matmul_stokes_rot         fortran/.../modules/mc_routines_general_mod.f90:1184-1242
#pragma once
#include <stdint.h>
#include "scene.h"

namespace monki {

template <typename T> struct Tol;
template <> struct Tol<float> {
    static constexpr float eps = 1.0e-16f;      // weight / probability / direction floor
    static constexpr float degenerate = 2.0e-7f;  // coplanar meridian test (float32 scale)
    static constexpr float vertical = 0.0f;       // |u| > 1 - vertical counts as vertical
    static constexpr float negligible = 0.0f;     // contributions below this are dropped
};
template <> struct Tol<double> {
    static constexpr double eps = 1.0e-16;
    static constexpr double degenerate = 1.0e-16;
    static constexpr double vertical = 1.0e-16;
    static constexpr double negligible = 1.0e-100;
};

template <typename T> __device__ __forceinline__ T pi_v() { return T(3.141592653589793); }

// ---------------------------------------------------------------------------------
// Philox4x32-10: counter (photon, round, draw block, 0), key (seed, 0).
// ---------------------------------------------------------------------------------
__device__ __forceinline__ uint4 philox4x32_10(uint4 c, uint2 k) {
#pragma unroll
    for (int r = 0; r < 10; ++r) {
        uint32_t hi0 = __umulhi(0xD2511F53u, c.x), lo0 = 0xD2511F53u * c.x;
        uint32_t hi1 = __umulhi(0xCD9E8D57u, c.z), lo1 = 0xCD9E8D57u * c.z;
        c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
        k.x += 0x9E3779B9u;
        k.y += 0xBB67AE85u;
    }
    return c;
}

struct PhotonStream {
    uint32_t photon, round, seed, block, lane;
    uint4 words;

    __device__ __forceinline__ void reset(uint32_t p, uint32_t r, uint32_t s) {
        photon = p; round = r; seed = s; block = 0; lane = 4;
    }
    // Uniform on the open float32 grid (w >> 9 + 0.5) * 2^-23: no log(0), never 1.
    __device__ __forceinline__ float next() {
        if (lane == 4) {
            words = philox4x32_10(make_uint4(photon, round, block++, 0u), make_uint2(seed, 0u));
            lane = 0;
        }
        uint32_t w = lane == 0 ? words.x : lane == 1 ? words.y : lane == 2 ? words.z : words.w;
        ++lane;
        return (float(w >> 9) + 0.5f) * 0x1p-23f;
    }
};

template <typename T> __device__ __forceinline__ T fsign(T a, T b) { return signbit(b) ? -fabs(a) : fabs(a); }

// ---------------------------------------------------------------------------------
// Scattering matrix elements. Phase matrices carry the /4 normalization of the
// reference (radiance normalized for incident E0 = pi).
// ---------------------------------------------------------------------------------
template <typename T>
struct Phase { T f11, f22, f33, f12, f34, f44; };  // f34, f44 only for nmat 4

template <typename T>
__device__ __forceinline__ Phase<T> rayleigh(T cs, T depol, int nmat) {
    T one_m = T(1) - cs * cs;
    T sin2 = one_m < Tol<T>::eps ? T(0) : one_m;
    T delta = (T(1) - depol) / (T(1) + depol / T(2));
    Phase<T> f;
    T diag = delta * (T(0.75) * (T(1) + cs * cs));
    f.f11 = (diag + (T(1) - delta)) / T(4);
    f.f22 = diag / T(4);
    f.f33 = delta * (T(1.5) * cs) / T(4);
    f.f12 = nmat > 1 ? delta * (T(-0.75) * sin2) / T(4) : T(0);
    // F44 = Delta' F33 with Delta' = (1 - 2 depol) / (1 - depol); Rayleigh has no F34.
    f.f34 = T(0);
    f.f44 = nmat > 3 ? (T(1) - T(2) * depol) / (T(1) - depol) * f.f33 : T(0);
    return f;
}

// Bracket of the ascending cosine table: an index guess from the uniform angle grid
// (as mie_scat_matrix does) corrected by a bounded walk. Returns lo (0-based) with
// cos[lo] <= cs <= cos[lo + 1], or lo = n - 1 when cs lands on the last node.
template <typename T>
__device__ __forceinline__ int lut_bracket(const T* __restrict__ cosv, int n, T cs) {
    T angle = acos(cs) / T(0.017453292519943295);
    int lo = int((T(180) - angle) / T(180) * T(n - 1));  // 0-based guess
    lo = lo < 0 ? 0 : (lo > n - 1 ? n - 1 : lo);
    if (lo == n - 1) return lo;
    for (int step = 0; step < 8 && lo > 0 && cs < __ldg(cosv + lo); ++step) --lo;
    for (int step = 0; step < 8 && lo < n - 2 && cs > __ldg(cosv + lo + 1); ++step) ++lo;
    return lo;
}

template <typename T>
__device__ __forceinline__ Phase<T> particle(const SceneView<T>& s, int sp, T cs, int nmat) {
    const int n = s.lut_n[sp];
    const T* __restrict__ cosv = s.lut_cos[sp];
    const T* __restrict__ f = s.lut_f[sp];
    int lo = lut_bracket(cosv, n, cs);
    Phase<T> r;
    if (lo == n - 1) {
        r.f11 = __ldg(f + 4 * lo); r.f22 = __ldg(f + 4 * lo + 1);
        r.f33 = __ldg(f + 4 * lo + 2); r.f12 = __ldg(f + 4 * lo + 3);
    } else {
        T x0 = __ldg(cosv + lo), x1 = __ldg(cosv + lo + 1);
        // linpol_dp_single: (y1 - y0) / (x1 - x0) * (xp - x0) + y0, exact at the nodes.
        auto lerp = [&](int e) {
            T y0 = __ldg(f + 4 * lo + e), y1 = __ldg(f + 4 * lo + 4 + e);
            if (cs == x1) return y1;
            if (cs == x0) return y0;
            return (y1 - y0) / (x1 - x0) * (cs - x0) + y0;
        };
        r.f11 = lerp(0); r.f22 = lerp(1); r.f33 = lerp(2); r.f12 = lerp(3);
    }
    r.f11 /= T(4); r.f22 /= T(4); r.f33 /= T(4);
    r.f12 = nmat > 1 ? r.f12 / T(4) : T(0);
    r.f34 = T(0); r.f44 = T(0);
    if (nmat > 3) {
        // {F34, F44} per node (version 3 tables), interpolated like the other elements.
        const T* __restrict__ v = s.lut_v[sp];
        if (lo == n - 1) {
            r.f34 = __ldg(v + 2 * lo); r.f44 = __ldg(v + 2 * lo + 1);
        } else {
            const T x0 = __ldg(cosv + lo), x1 = __ldg(cosv + lo + 1);
            auto lerp = [&](int e) {
                T y0 = __ldg(v + 2 * lo + e), y1 = __ldg(v + 2 * lo + 2 + e);
                if (cs == x1) return y1;
                if (cs == x0) return y0;
                return (y1 - y0) / (x1 - x0) * (cs - x0) + y0;
            };
            r.f34 = lerp(0); r.f44 = lerp(1);
        }
        r.f34 /= T(4); r.f44 /= T(4);
    }
    return r;
}

template <typename T>
__device__ __forceinline__ Phase<T> phase(const SceneView<T>& s, int sp, T cs, int nmat) {
    return sp < 0 ? rayleigh<T>(cs, s.depol, nmat) : particle<T>(s, sp, cs, nmat);
}

// ---------------------------------------------------------------------------------
// Meridian-plane rotation: returns {C1, S1, C2, S2} with L(2,2) = L(3,3) = C and
// L(3,2) = S for the incident (L1) and scattered (L2) rotations.
// ---------------------------------------------------------------------------------
template <typename T>
struct Rot { T c1, s1, c2, s2; };

// The rotations with the sines and cosines of both azimuths supplied by the caller.
template <typename T>
__device__ __forceinline__ Rot<T> rotation_pre(T cs, T uo, T u1, T phio, T phi1, T cpo, T spo, T cp1, T sp1) {
    Rot<T> r{T(1), T(0), T(1), T(0)};
    const T pi = pi_v<T>();
    T dphi = fabs(phio - phi1);
    T rem = fmod(dphi, pi);
    if (rem < Tol<T>::degenerate || fabs(rem - pi) < Tol<T>::degenerate) return r;
    const T vert = T(1) - Tol<T>::vertical;
    bool vo = fabs(uo) > vert || fabs(uo) >= T(1);
    bool v1 = fabs(u1) > vert || fabs(u1) >= T(1);
    if (vo && v1) return r;
    T fac = T(1) - uo * uo;
    T sino = fac < Tol<T>::eps ? T(0) : sqrt(fac);
    fac = T(1) - u1 * u1;
    T sin1 = fac < Tol<T>::eps ? T(0) : sqrt(fac);
    T cosi1, cosi2, q;
    if (v1) {
        cosi1 = fsign(T(1), u1);
        cosi2 = -cosi1 * (cp1 * cpo + sp1 * spo);
        q = (sino * spo) * cp1 - (sino * cpo) * sp1;
    } else if (vo) {
        cosi2 = fsign(T(1), uo);
        cosi1 = -cosi2 * (cp1 * cpo + sp1 * spo);
        q = spo * (sin1 * cp1) - cpo * (sin1 * sp1);
    } else {
        T eps = Tol<T>::eps;
        T d1 = (T(1) - uo * uo) * (T(1) - cs * cs);
        T d2 = (T(1) - u1 * u1) * (T(1) - cs * cs);
        cosi1 = (u1 - uo * cs) / sqrt(d1 > eps ? d1 : eps);
        cosi2 = (uo - u1 * cs) / sqrt(d2 > eps ? d2 : eps);
        q = (sino * spo) * (sin1 * cp1) - (sino * cpo) * (sin1 * sp1);
    }
    // Near-degenerate geometry can push the rounded cosines past +-1; without the clamp
    // C = cos^2 would exceed 1 and the rotation would amplify Q and U (in FP32 often).
    cosi1 = fmin(T(1), fmax(T(-1), cosi1));
    cosi2 = fmin(T(1), fmax(T(-1), cosi2));
    fac = T(1) - cosi1 * cosi1;
    T sini1 = fac < Tol<T>::eps ? T(0) : sqrt(fac) * fsign(T(1), q);
    fac = T(1) - cosi2 * cosi2;
    T sini2 = fac < Tol<T>::eps ? T(0) : sqrt(fac) * fsign(T(1), q);
    r.c1 = cosi1 * cosi1 - sini1 * sini1;
    r.s1 = T(2) * sini1 * cosi1;
    r.c2 = cosi2 * cosi2 - sini2 * sini2;
    r.s2 = T(2) * sini2 * cosi2;
    return r;
}

template <typename T>
__device__ __forceinline__ Rot<T> rotation(T cs, T uo, T u1, T phio, T phi1) {
    T cpo, spo, cp1, sp1;
    sincos(phio, &spo, &cpo);
    sincos(phi1, &sp1, &cp1);
    return rotation_pre<T>(cs, uo, u1, phio, phi1, cpo, spo, cp1, sp1);
}

// S_out = L2 * F * L1 * S (matmul_stokes_rot followed by the forward-mode product). The
// scattering matrix has F(3,4) = F34 and F(4,3) = -F34, so the rotated phase matrix has
// P(2,4) = -S2 F34, P(3,4) = C2 F34, P(4,2) = -S1 F34, P(4,3) = -C1 F34, P(4,4) = F44.
template <typename T>
__device__ __forceinline__ void scatter_stokes(const Phase<T>& f, const Rot<T>& r, int nmat,
                                               const T* s, T* out) {
    if (nmat == 1) { out[0] = f.f11 * s[0]; return; }
    const T C1 = r.c1, S1 = r.s1, C2 = r.c2, S2 = r.s2;
    out[0] = f.f11 * s[0] + f.f12 * C1 * s[1] - f.f12 * S1 * s[2];
    out[1] = C2 * f.f12 * s[0] + (C1 * C2 * f.f22 - S1 * S2 * f.f33) * s[1] +
             (-C2 * S1 * f.f22 - C1 * S2 * f.f33) * s[2];
    out[2] = S2 * f.f12 * s[0] + (C1 * S2 * f.f22 + C2 * S1 * f.f33) * s[1] +
             (C1 * C2 * f.f33 - S1 * S2 * f.f22) * s[2];
    if (nmat > 3) {
        out[1] += -S2 * f.f34 * s[3];
        out[2] += C2 * f.f34 * s[3];
        out[3] = -S1 * f.f34 * s[1] - C1 * f.f34 * s[2] + f.f44 * s[3];
    }
}

// The rotated phase matrix P = L2 F L1 of matmul_stokes_rot, row-major nmat x nmat.
template <typename T>
__device__ __forceinline__ void phase_matrix(const Phase<T>& f, const Rot<T>& r, int nmat, T P[4][4]) {
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) P[a][b] = T(0);
    P[0][0] = f.f11;
    if (nmat == 1) return;
    const T C1 = r.c1, S1 = r.s1, C2 = r.c2, S2 = r.s2;
    P[0][1] = f.f12 * C1;
    P[0][2] = -f.f12 * S1;
    P[1][0] = C2 * f.f12;
    P[1][1] = C1 * C2 * f.f22 - S1 * S2 * f.f33;
    P[1][2] = -C2 * S1 * f.f22 - C1 * S2 * f.f33;
    P[2][0] = S2 * f.f12;
    P[2][1] = C1 * S2 * f.f22 + C2 * S1 * f.f33;
    P[2][2] = C1 * C2 * f.f33 - S1 * S2 * f.f22;
    if (nmat > 3) {
        P[1][3] = -S2 * f.f34;
        P[2][3] = C2 * f.f34;
        P[3][1] = -S1 * f.f34;
        P[3][2] = -C1 * f.f34;
        P[3][3] = f.f44;
    }
}

// Spherical trigonometry after an accepted (cos_sca, sigma) sample.
template <typename T>
__device__ __forceinline__ void outgoing(T cos_in, T cos_sca, T sigma, T& cos_out, T& dphi) {
    const T eps = Tol<T>::eps;
    T a = T(1) - cos_in * cos_in, b = T(1) - cos_sca * cos_sca;
    T sin_in = sqrt(a > eps ? a : eps);
    T sin_sca = sqrt(b > eps ? b : eps);
    cos_out = cos_in * cos_sca + sin_in * sin_sca * cos(sigma);
    T c = T(1) - cos_out * cos_out;
    T sin_out = sqrt(c > eps ? c : eps);
    T frac = (cos_sca - cos_in * cos_out) / (sin_in * sin_out);
    if (frac >= T(1) - eps) dphi = T(0);
    else if (frac <= T(-1) + eps) dphi = pi_v<T>();
    else dphi = acos(frac) * fsign(T(1), sigma);
    dphi = -dphi;
}

// Draw a bracket of the bound CDF with the guide table, then interpolate the cosine.
template <typename T>
__device__ __forceinline__ T sample_cdf(const SceneView<T>& s, int sp, T u) {
    const int n = s.lut_n[sp];
    const T* __restrict__ cdf = s.lut_cdf[sp];
    const T* __restrict__ cosv = s.lut_cos[sp];
    int g = int(u * T(kGuide));
    g = g < 0 ? 0 : (g > kGuide ? kGuide : g);
    int lo = __ldg(s.guide[sp] + g);
    while (lo < n - 2 && __ldg(cdf + lo + 1) < u) ++lo;
    T x0 = __ldg(cdf + lo), x1 = __ldg(cdf + lo + 1);
    T y0 = __ldg(cosv + lo), y1 = __ldg(cosv + lo + 1);
    if (u == x1) return y1;
    if (u == x0) return y0;
    return (y1 - y0) / (x1 - x0) * (u - x0) + y0;
}

// Polarized rejection sampling: pdf F11 + F12 (Q cos 2 sigma + sign U sin 2 sigma) with
// sign -1 forward and +1 backward. Rayleigh: uniform cosine with the F11(0 deg) bound;
// particles: bound F11 + |F12| drawn from its CDF. Capped at 4096.
template <typename T, typename Stream>
__device__ __forceinline__ bool sample_direction(const SceneView<T>& s, int sp, int nmat, const T* st,
                                                 T cos_in, Stream& rng, T& cos_out, T& dphi,
                                                 T& cos_sca, T sign = T(-1)) {
    const T pi = pi_v<T>();
    const T bound_gas = rayleigh<T>(T(1), s.depol, 1).f11;
    for (int attempt = 0; attempt < 4096; ++attempt) {
        T u1 = T(rng.next());
        T cs = sp < 0 ? T(2) * u1 - T(1) : sample_cdf<T>(s, sp, u1);
        T sigma = T(2) * pi * T(rng.next()) - pi;
        Phase<T> f = phase<T>(s, sp, cs, nmat);
        T pdf = f.f11;
        if (nmat > 1) {
            T s2, c2;
            sincos(T(2) * sigma, &s2, &c2);
            pdf = f.f11 + f.f12 * (st[1] * c2 + sign * st[2] * s2);
        }
        T bound = sp < 0 ? bound_gas : f.f11 + fabs(f.f12);
        if (T(rng.next()) * bound > pdf) continue;
        cos_sca = cs;
        outgoing<T>(cos_in, cs, sigma, cos_out, dphi);
        return true;
    }
    return false;
}

}  // namespace monki
