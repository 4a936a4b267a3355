// Photon-history megakernel and per-round FP64 flush for MONKI transport on sm_103a.
//
// One thread carries one photon history at a time and pulls the next photon of the
// round group from a grid-stride sequence until the group is exhausted, so a warp
// stays busy while its histories have very different lengths. The per-photon random
// stream depends only on (seed, round, photon), never on the launch shape.
//
// Reference control flow: fortran/monki/upstream/PROGRAM/mc.f90:314-1436 (labels
// 1000/1010/1020/3000/4000), ADVANCE_internal mc.f90:1531-1580, and the detector
// estimators calc_radiances_pol / calc_radiances_and_paths_pol
// (modules/mc_routines_cartesian_mod.f90:37-393, 849-1222).
#pragma once
#include "physics.cuh"

namespace monki {

template <typename TA>
__device__ __forceinline__ void tally_add(TA* p, TA v) { atomicAdd(p, v); }

// Per-thread history of the photon's path length per layer (the AMF path_layers).
template <typename T>
struct History { T len[kMaxLayers]; };

// One step of the cell walk (ADVANCE): move to the nearest face in the current
// direction; x before y before z on ties; periodic in x and y.
template <typename T>
__device__ __forceinline__ T advance(const SceneView<T>& s, int& i, int& j, int& k, T& x, T& y, T& z,
                                     int is, int js, int ks, T aa, T ba, T ca, T ai, T bi, T ci) {
    T dx = x * ai, dy = y * bi, dz = z * ci;
    T dist = fmin(dx, fmin(dy, dz));
    if (dx == dist) {
        i += is; i = i < 0 ? i + s.nx : (i >= s.nx ? i - s.nx : i);
        x = s.xunit;
        y = fmax(T(0), y - ba * dist);
        z = fmax(T(0), z - ca * dist);
    } else if (dy == dist) {
        j += js; j = j < 0 ? j + s.ny : (j >= s.ny ? j - s.ny : j);
        x = fmax(T(0), x - aa * dist);
        y = s.yunit;
        z = fmax(T(0), z - ca * dist);
    } else {
        k += ks;
        x = fmax(T(0), x - aa * dist);
        y = fmax(T(0), y - ba * dist);
        if (k >= 0 && k < s.nz) z = __ldg(s.zunit + k);
    }
    return dist;
}

template <typename T>
__device__ __forceinline__ T beta_at(const SceneView<T>& s, int i, int j, int k) {
    return __ldg(s.cells + 4 * (i + s.nx * (j + s.ny * k)));
}

// Peel-off of one event towards view ia: optical depth along the view ray (explicit
// cell walk through horizontally varying layers, then the uniform-layer prefix), the
// register pixel from the analytic top-of-atmosphere projection, and the Stokes /
// weighted-path / weight tallies. Returns false when the ray exceeds the step cap.
template <typename T, typename TA, int NMAT, bool PATHS>
__device__ __forceinline__ bool detector(const SceneView<T>& s, int ia, const T* prob, int i0, int j0, int k0,
                                         T x0, T y0, T z0, T a0, T b0, T c0, const History<T>& hist,
                                         TA* bank, const TallyLayout& L, uint32_t max_steps,
                                         uint64_t& visits, uint64_t& updates) {
    const T eps = Tol<T>::eps;
    const T a = s.va[ia], b = s.vb[ia], c = s.vc[ia];
    T x = x0, y = y0, z = z0;
    if (a * a0 < T(0)) x = fmax(T(0), s.xunit - x);
    if (b * b0 < T(0)) y = fmax(T(0), s.yunit - y);
    if (c * c0 < T(0)) z = fmax(T(0), __ldg(s.zunit + k0) - z);
    const int is = signbit(a) ? -1 : 1, js = signbit(b) ? -1 : 1, ks = signbit(c) ? -1 : 1;
    const T aa = fabs(a), ba = fabs(b), ca = fabs(c);
    const T ai = T(1) / fmax(aa, eps), bi = T(1) / fmax(ba, eps), ci = T(1) / fmax(ca, eps);
    const T x_old = x, y_old = y, z_old = z;
    const int top = s.nz - 1;  // first non-physical (vacuum) layer
    T tau = T(0);
    int i = i0, j = j0, k = k0;
    uint32_t steps = 0;
    while (k >= 0 && k < top) {
        if (k >= s.uniform_top) {
            // Every layer from k up is horizontally uniform: the remaining slant optical
            // depth is the vertical prefix divided by the view cosine.
            tau += (z * beta_at(s, i, j, k) + __ldg(s.tau_above + k)) * ci;
            ++visits;
            break;
        }
        if (++steps > max_steps) return false;
        T bv = beta_at(s, i, j, k);
        T dist = advance(s, i, j, k, x, y, z, is, js, ks, aa, ba, ca, ai, bi, ci);
        tau += dist * bv;
        ++visits;
    }
    // Register grid (k_register == k_detector == top): project the event to the top of
    // the physical atmosphere.
    T height = __ldg(s.zsum + k0) + (ks > 0 ? __ldg(s.zunit + k0) - z_old : z_old);
    height = __ldg(s.zsum + top) - height;
    T dxp = aa * height / ca, dyp = ba * height / ca;
    int di = int(((s.xunit - x_old) + dxp) / s.xunit);
    int dj = int(((s.yunit - y_old) + dyp) / s.yunit);
    int pi_ = (i0 + is * (di % s.nx)) % s.nx; pi_ = pi_ < 0 ? pi_ + s.nx : pi_;
    int pj_ = (j0 + js * (dj % s.ny)) % s.ny; pj_ = pj_ < 0 ? pj_ + s.ny : pj_;
    const T att = exp(-tau);
    const uint32_t pixel = uint32_t(pi_ + s.nx * (pj_ + s.ny * ia));
#pragma unroll
    for (int m = 0; m < NMAT; ++m) tally_add(bank + NMAT * pixel + m, TA(prob[m] * att));
    updates += NMAT;
    if (PATHS) {
        const T w = prob[0] * att;
        TA* paths = bank + L.stokes + size_t(pixel) * s.nz;
        // Ray length per layer: the partial event layer, then whole layers above it.
        // (The cell walk's segment sums equal these vertical extents over the cosine.)
        for (int kk = 0; kk < s.nz; ++kk) {
            T ang = kk < k0 || kk >= top ? T(0) : (kk == k0 ? z_old * ci : __ldg(s.zunit + kk) * ci);
            T v = w * (hist.len[kk] + ang);
            if (v != T(0)) { tally_add(paths + kk, TA(v)); ++updates; }
        }
        tally_add(bank + L.stokes + L.paths + pixel, TA(w));
        ++updates;
    }
    return true;
}

template <typename T, typename TA, int NMAT, bool PATHS>
__global__ void __launch_bounds__(256)
transport_kernel(SceneView<T> s, Controls ctl, TA* __restrict__ banks, TallyLayout L,
                 uint32_t* __restrict__ failure, unsigned long long* __restrict__ counters) {
    const T eps = Tol<T>::eps;
    const T pi = pi_v<T>();
    const uint32_t stride = gridDim.x * blockDim.x;
    const uint32_t tid = blockIdx.x * blockDim.x + threadIdx.x;
    const uint32_t warp = tid >> 5;
    const uint32_t ncol = uint32_t(s.nx * s.ny);
    const int top = s.nz - 1;
    uint64_t scatters = 0, visits_fp = 0, visits_det = 0, updates = 0;
    History<T> hist;
    PhotonStream rng;

    for (uint32_t n = tid; n < ctl.count; n += stride) {
        const uint32_t identity = ctl.first + n;
        const uint32_t round_offset = identity / ctl.per_round;
        const uint32_t photon = identity % ctl.per_round;
        TA* bank = banks + (size_t(round_offset) * L.shards + (warp % L.shards)) * L.count;
        rng.reset(photon, ctl.first_round + round_offset, ctl.seed);
        const uint32_t column = photon % ncol;
        int i = int(column % uint32_t(s.nx)), j = int(column / uint32_t(s.nx));
        if (j > s.ny - 1) j = s.ny - 1;
        int k = top;
        T x = s.xunit * T(rng.next());
        T y = s.yunit * T(rng.next());
        T z = __ldg(s.zunit + k);
        T st[3] = {T(1), T(0), T(0)};
        T weight = T(1);
        if (PATHS) for (int kk = 0; kk < s.nz; ++kk) hist.len[kk] = T(0);
        T a = s.a0, b = s.b0, c = s.c0, phi = s.phi0;
        T remains = T(0);
        bool new_path = true;
        uint32_t steps = 0, flag = 0;
        for (;;) {
            if (new_path) remains = -log(fmax(T(rng.next()), eps));
            new_path = false;
            const int is = signbit(a) ? -1 : 1, js = signbit(b) ? -1 : 1, ks = signbit(c) ? -1 : 1;
            const T aa = fabs(a), ba = fabs(b), ca = fabs(c);
            const T ai = T(1) / fmax(aa, eps), bi = T(1) / fmax(ba, eps), ci = T(1) / fmax(ca, eps);
            bool surface = false, escaped = false;
            for (;;) {
                if (++steps > ctl.max_steps) { flag = kHistoryCap; break; }
                ++visits_fp;
                T bv = (k < top && k >= 0) ? beta_at(s, i, j, k) : T(0);
                if (bv > eps) {
                    T de = remains / bv;
                    if (de < x * ai && de < y * bi && de < z * ci) {
                        x = fmax(T(0), x - aa * de);
                        y = fmax(T(0), y - ba * de);
                        z = fmax(T(0), z - ca * de);
                        if (PATHS) hist.len[k] += de;
                        break;  // atmospheric event
                    }
                }
                const int k_old = k;
                T dist = advance(s, i, j, k, x, y, z, is, js, ks, aa, ba, ca, ai, bi, ci);
                if (PATHS) hist.len[k_old] += dist;
                remains -= dist * bv;
                if (k >= 0 && k <= top) continue;
                if (k > top) { escaped = true; break; }
                surface = true;
                break;
            }
            if (flag || escaped) break;
            T prob[3];
            if (surface) {
                const T a_int = a, b_int = b, c_int = c;
                k = 0;
                z = T(0);
                weight *= __ldg(s.albedo + i + s.nx * j);
                if (weight < eps) break;
                ++scatters;
                for (int ia = 0; ia < s.angles; ++ia) {
                    prob[0] = s.vc[ia] > T(0) ? st[0] * s.vc[ia] * weight : T(0);
                    prob[1] = T(0); prob[2] = T(0);
                    if (!isfinite(prob[0])) { flag = kNonfinite; break; }
                    if (!(prob[0] > eps)) continue;
                    if (!detector<T, TA, NMAT, PATHS>(s, ia, prob, i, j, k, x, y, z, a_int, b_int, c_int, hist,
                                                      bank, L, ctl.max_steps, visits_det, updates)) {
                        flag = kDetectorCap; break;
                    }
                }
                if (flag) break;
                // Lambertian reflection (GROUND_LAMB2): mu = sqrt(P), phi = 2 pi U.
                T P = T(rng.next()), U = T(rng.next());
                T mu = sqrt(P);
                T phi_out = T(2) * pi * U;
                T sine = sqrt(fmax(T(0), T(1) - mu * mu));
                T sp, cp;
                sincos(phi_out, &sp, &cp);
                a = sine * cp; b = sine * sp; c = fabs(mu);
                st[1] = T(0); st[2] = T(0);
                if (a * a_int < T(0)) x = fmax(T(0), s.xunit - x);
                if (b * b_int < T(0)) y = fmax(T(0), s.yunit - y);
                if (c * c_int < T(0)) z = fmax(T(0), __ldg(s.zunit + k) - z);
                phi = phi_out;
                continue;  // keep the remaining optical path (GOTO 1010)
            }
            // Atmospheric event: species by cumulative extinction fraction; gas last.
            const T rtemp = T(rng.next());
            int sp = -1;
            {
                const T* cell = s.cells + 4 * (i + s.nx * (j + s.ny * k));
                for (int q = 0; q < s.ntypes; ++q)
                    if (__ldg(cell + 1 + q) > rtemp) { sp = q; break; }
            }
            weight *= sp < 0 ? __ldg(s.ssalb_gas + k) : s.ssalb_aer[sp];
            if (weight < eps) break;
            ++scatters;
            for (int ia = 0; ia < s.angles; ++ia) {
                const T vc = s.vc[ia];
                T cs = c * vc + sqrt(fmax(eps, T(1) - c * c)) * sqrt(fmax(eps, T(1) - vc * vc)) *
                                    cos(phi - s.vphi[ia]);
                Rot<T> r = NMAT > 1 ? rotation<T>(cs, c, vc, phi, s.vphi[ia]) : Rot<T>{T(1), T(0), T(1), T(0)};
                Phase<T> f = phase<T>(s, sp, cs, NMAT);
                T back[3];
                scatter_stokes<T>(f, r, NMAT, st, back);
                for (int m = 0; m < NMAT; ++m) prob[m] = back[m] * weight;
                if (prob[0] < Tol<T>::negligible) for (int m = 0; m < NMAT; ++m) prob[m] = T(0);
                bool finite = true;
                for (int m = 0; m < NMAT; ++m) finite = finite && isfinite(prob[m]);
                if (!finite) { flag = kNonfinite; break; }
                if (!(prob[0] > eps)) continue;
                if (!detector<T, TA, NMAT, PATHS>(s, ia, prob, i, j, k, x, y, z, a, b, c, hist, bank, L,
                                                  ctl.max_steps, visits_det, updates)) {
                    flag = kDetectorCap; break;
                }
            }
            if (flag) break;
            T cos_out, dphi, cos_sca;
            if (!sample_direction<T>(s, sp, NMAT, st, c, rng, cos_out, dphi, cos_sca)) {
                flag = kSamplingCap; break;
            }
            const T phi_out = phi + dphi;
            {
                Rot<T> r = NMAT > 1 ? rotation<T>(cos_sca, c, cos_out, phi, phi_out) : Rot<T>{T(1), T(0), T(1), T(0)};
                Phase<T> f = phase<T>(s, sp, cos_sca, NMAT);
                T ns[3];
                scatter_stokes<T>(f, r, NMAT, st, ns);
                const T s0 = ns[0];
                for (int m = 0; m < NMAT; ++m) st[m] = ns[m] / s0;
                if (st[0] < Tol<T>::negligible) for (int m = 0; m < NMAT; ++m) st[m] = T(0);
                bool ok = true;
                for (int m = 0; m < NMAT; ++m) ok = ok && isfinite(st[m]);
                if (NMAT == 3 && ok) ok = sqrt(st[1] * st[1] + st[2] * st[2]) <= st[0] + T(1e-2);
                if (!ok) { flag = kInvalidStokes; break; }
            }
            const T a_bak = a, b_bak = b, c_bak = c;
            {
                T so = sqrt(fmax(T(0), T(1) - cos_out * cos_out));
                T spo, cpo;
                sincos(phi_out, &spo, &cpo);
                a = cpo * so; b = spo * so; c = cos_out;
            }
            if (a * a_bak < T(0)) x = fmax(T(0), s.xunit - x);
            if (b * b_bak < T(0)) y = fmax(T(0), s.yunit - y);
            if (c * c_bak < T(0)) z = fmax(T(0), __ldg(s.zunit + k) - z);
            phi = phi_out;
            new_path = true;
        }
        if (flag) atomicOr(failure, flag);
    }
    // Warp-aggregated counters: scatters, free-path visits, detector visits, tally updates.
    unsigned long long v0 = scatters, v1 = visits_fp, v2 = visits_det, v3 = updates;
#pragma unroll
    for (int off = 16; off > 0; off >>= 1) {
        v0 += __shfl_down_sync(0xffffffffu, v0, off);
        v1 += __shfl_down_sync(0xffffffffu, v1, off);
        v2 += __shfl_down_sync(0xffffffffu, v2, off);
        v3 += __shfl_down_sync(0xffffffffu, v3, off);
    }
    if ((threadIdx.x & 31) == 0) {
        atomicAdd(counters + 0, v0);
        atomicAdd(counters + 1, v1);
        atomicAdd(counters + 2, v2);
        atomicAdd(counters + 3, v3);
    }
}

// Sum the shards of every round in FP64, apply mu0/mu to Stokes (mc.f90:1456-1474),
// write RawTallies order (stokes(nmat,nx,ny,angles), paths(nx,ny,nz,angles),
// weights(nx,ny,angles), Fortran order) and clear the banks for the next group.
template <typename TA>
__global__ void flush_kernel(TA* __restrict__ banks, TallyLayout L, int nmat, int nx, int ny, int nz,
                             int angles, const double* __restrict__ mu0mu, uint32_t rounds,
                             double* __restrict__ out) {
    const uint32_t per_round = L.count;
    const uint64_t total = uint64_t(per_round) * rounds;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < total;
         e += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t r = uint32_t(e / per_round);
        const uint32_t o = uint32_t(e % per_round);  // output (Fortran-order) index
        uint32_t src;
        double scale = 1.0;
        if (o < L.stokes) {
            src = o;  // identical layout
            uint32_t ia = o / uint32_t(nmat * nx * ny);
            scale = mu0mu[ia];
        } else if (o < L.stokes + L.paths) {
            uint32_t q = o - L.stokes;  // i + nx*(j + ny*(k + nz*ia))
            uint32_t i = q % nx, t = q / nx;
            uint32_t j = t % ny; t /= ny;
            uint32_t k = t % nz, ia = t / nz;
            src = L.stokes + k + nz * (i + nx * (j + ny * ia));
        } else {
            src = o;
        }
        double acc = 0.0;
        TA* base = banks + size_t(r) * L.shards * per_round + src;
        for (uint32_t sh = 0; sh < L.shards; ++sh) {
            acc += double(base[size_t(sh) * per_round]);
            base[size_t(sh) * per_round] = TA(0);
        }
        out[e] = acc * scale;
    }
}

}  // namespace monki
