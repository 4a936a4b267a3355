// FP64 round statistics on the device.
//
// After each round group's flush, the per-round tallies (RawTallies order) are folded
// into device accumulators in round order, with the operations of the reference driver
// and stopping rules (python/monki/simulation.py:86-103, python/monki/convergence.py:
// 37-99), each correctly rounded in FP64 (no fused multiply-add), so the host receives
// the same sums it would have formed from the tallies:
//
//   stokes   total += x;  n = x / ppc;  sum += n;  squares += n * n
//   paths    sum += p;    Welford moments of p and of the pixel weight w with
//            count c:  dp = p - mp; dw = w - mw; mp += dp / c; mw += dw / c;
//                      m2p += dp (p - mp); m2w += dw (w - mw); cov += dp (w - mw)
//   weights  sum += w;    mw, m2w as above
//
// Layout (doubles): total[S] sum[S] squares[S] | paths[P] mean[P] m2[P] cov[P] |
// weights[W] mean[W] m2[W], with S = nmat pixels, P = pixels nz (vacuum layer included;
// the stopping rule ignores it), W = pixels, pixels = nx ny angles.
#pragma once
#include <stdint.h>
#include <stddef.h>

namespace monki {

struct StatsLayout {
    uint32_t stokes, paths, weights;
    uint32_t nx, ny, nz;
    size_t count;
};

// phase 0: Stokes and path elements (reading the weight moments of the previous groups);
// phase 1: weight elements. One thread per element, rounds in order.
__global__ void stats_update(const double* __restrict__ out, uint32_t count, uint32_t rounds, uint32_t before,
                             StatsLayout L, double ppc, double* __restrict__ stats, int phase) {
    const uint32_t S = L.stokes, P = L.paths, W = L.weights;
    double* total = stats;
    double* sum = stats + S;
    double* squares = stats + 2 * size_t(S);
    double* psum = stats + 3 * size_t(S);
    double* pmean = psum + P;
    double* pm2 = pmean + P;
    double* pcov = pm2 + P;
    double* wsum = pcov + P;
    double* wmean = wsum + W;
    double* wm2 = wmean + W;
    const uint32_t elements = phase == 0 ? S + P : W;
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < elements; e += gridDim.x * blockDim.x) {
        if (phase == 0 && e < S) {
            double t = total[e], s = sum[e], q = squares[e];
            for (uint32_t r = 0; r < rounds; ++r) {
                const double x = out[size_t(r) * count + e];
                t = __dadd_rn(t, x);
                const double n = __ddiv_rn(x, ppc);
                s = __dadd_rn(s, n);
                q = __dadd_rn(q, __dmul_rn(n, n));
            }
            total[e] = t; sum[e] = s; squares[e] = q;
        } else if (phase == 0) {
            const uint32_t q = e - S;
            const uint32_t i = q % L.nx, rest = q / L.nx;
            const uint32_t j = rest % L.ny, rest2 = rest / L.ny;
            const uint32_t ia = rest2 / L.nz;
            const uint32_t pixel = i + L.nx * (j + L.ny * ia);
            double ps = psum[q], mp = pmean[q], m2p = pm2[q], cov = pcov[q], mw = wmean[pixel];
            for (uint32_t r = 0; r < rounds; ++r) {
                const double p = out[size_t(r) * count + S + q];
                const double w = out[size_t(r) * count + S + P + pixel];
                const double c = double(before + r + 1);
                ps = __dadd_rn(ps, p);
                const double dp = __dsub_rn(p, mp), dw = __dsub_rn(w, mw);
                mp = __dadd_rn(mp, __ddiv_rn(dp, c));
                mw = __dadd_rn(mw, __ddiv_rn(dw, c));
                m2p = __dadd_rn(m2p, __dmul_rn(dp, __dsub_rn(p, mp)));
                cov = __dadd_rn(cov, __dmul_rn(dp, __dsub_rn(w, mw)));
            }
            psum[q] = ps; pmean[q] = mp; pm2[q] = m2p; pcov[q] = cov;
        } else {
            double ws = wsum[e], mw = wmean[e], m2w = wm2[e];
            for (uint32_t r = 0; r < rounds; ++r) {
                const double w = out[size_t(r) * count + S + P + e];
                const double c = double(before + r + 1);
                ws = __dadd_rn(ws, w);
                const double dw = __dsub_rn(w, mw);
                mw = __dadd_rn(mw, __ddiv_rn(dw, c));
                m2w = __dadd_rn(m2w, __dmul_rn(dw, __dsub_rn(w, mw)));
            }
            wsum[e] = ws; wmean[e] = mw; wm2[e] = m2w;
        }
    }
}

// history[r * nmat + m] = sum over pixels of the round's normalized Stokes element m, in a
// fixed order (strided partial sums, then a shared-memory tree). Grid (rounds, nmat).
__global__ void round_sums(const double* __restrict__ out, uint32_t count, uint32_t nmat, uint32_t stokes,
                           double ppc, double* __restrict__ history) {
    __shared__ double part[256];
    const uint32_t r = blockIdx.x, m = blockIdx.y;
    const uint32_t pixels = stokes / nmat;
    double acc = 0.0;
    for (uint32_t px = threadIdx.x; px < pixels; px += blockDim.x)
        acc = __dadd_rn(acc, __ddiv_rn(out[size_t(r) * count + m + nmat * px], ppc));
    part[threadIdx.x] = acc;
    __syncthreads();
    for (uint32_t half = blockDim.x / 2; half > 0; half >>= 1) {
        if (threadIdx.x < half) part[threadIdx.x] = __dadd_rn(part[threadIdx.x], part[threadIdx.x + half]);
        __syncthreads();
    }
    if (threadIdx.x == 0) history[size_t(r) * nmat + m] = part[0];
}

}  // namespace monki
