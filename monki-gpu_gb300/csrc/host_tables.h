// Host side of the transport tables: the session settings string, the prepared table
// stream (transport.bin v1 of kernels/cpu/worker.f90:1102-1120; v2 adds one view azimuth
// per view, v3 the F34 / F44 tables), its packing into one device allocation and the
// SceneView of that allocation. Shared by the single-scene session (session.cu) and the
// multi-scene session (multi.cu).
#pragma once
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <vector>

#include "wavefront.cuh"

namespace monki {
namespace host {


constexpr double kDegToRad = 0.017453292519943295;

struct Config {
    bool fp64 = false;
    bool wavefront = true;       // engine=wavefront (default) or engine=megakernel
    uint32_t shards = 8;
    int block = 256;
    int blocks_per_sm = 0;       // 0 = occupancy-derived
    bool uniform_prefix = true;
    uint32_t pool = 1u << 22;    // wavefront photon slots (4 Mi: +4 % over 1 Mi on the box cloud)
    uint32_t check_every = 8;    // wavefront iterations between host checks
    // Walk steps per photon per launch. A walk that runs out pauses and resumes in the next
    // launch, where the paused walks fill warps of their own: short budgets keep the lanes of
    // a warp in step (box cloud: 2.76 G scatters/s at 24, 2.84 at 3, 2.83 at 2).
    uint32_t walk = 3;
    double epsilon = 0.0;        // guided: detector-branch probability at particle scatters
    double roulette = 0.0;       // guided: roulette weight (0 = off)
    double cap = 0.0;            // guided: detector branch only below this weight (0 = always)
    double split = 0.0;          // guided: split above split x the roulette weight (0 = off)
    bool importance = false;     // tally per-cell importance (pilot runs)
    bool graphs = true;          // replay each batch of wavefront iterations as a CUDA graph
    bool orders = false;         // scattering-order diagnostics (single scattering, locations)
    bool rectangles = true;      // cross equal-extinction rectangles of the band in one step
    uint32_t tail = 1u << 16;    // run a group's last photons to their end in one launch below this many (0 = off)
    int fused = -1;              // 1: scatter and walk in one step kernel; 0: separate kernels; -1: by scene
};

inline Config parse_config(const char* text) {
    Config c;
    if (!text) return c;
    std::string s(text);
    size_t pos = 0;
    while (pos < s.size()) {
        size_t end = s.find_first_of(",;", pos);
        if (end == std::string::npos) end = s.size();
        std::string item = s.substr(pos, end - pos);
        pos = end + 1;
        if (item.empty()) continue;
        size_t eq = item.find('=');
        if (eq == std::string::npos) throw std::runtime_error("Malformed config item: " + item);
        std::string key = item.substr(0, eq), value = item.substr(eq + 1);
        auto as_int = [&](long lo, long hi) {
            char* e = nullptr;
            long v = std::strtol(value.c_str(), &e, 10);
            if (!e || *e || v < lo || v > hi) throw std::runtime_error("Invalid config value: " + item);
            return v;
        };
        if (key == "precision") {
            if (value == "fp32") c.fp64 = false;
            else if (value == "fp64") c.fp64 = true;
            else throw std::runtime_error("precision must be fp32 or fp64");
        } else if (key == "shards") c.shards = uint32_t(as_int(1, 64));
        else if (key == "block") c.block = int(as_int(32, 256));
        else if (key == "blocks_per_sm") c.blocks_per_sm = int(as_int(0, 64));
        else if (key == "uniform_prefix") c.uniform_prefix = as_int(0, 1) != 0;
        else if (key == "engine") {
            if (value == "wavefront") c.wavefront = true;
            else if (value == "megakernel") c.wavefront = false;
            else throw std::runtime_error("engine must be wavefront or megakernel");
        } else if (key == "pool") c.pool = uint32_t(as_int(1024, 1l << 26));
        else if (key == "check_every") c.check_every = uint32_t(as_int(1, 1024) + 1) & ~1u;  // even: see run_wavefront
        else if (key == "walk") c.walk = uint32_t(as_int(1, 1 << 20));
        else if (key == "epsilon" || key == "roulette" || key == "cap" || key == "split") {
            char* e = nullptr;
            const double v = std::strtod(value.c_str(), &e);
            if (!e || *e || !std::isfinite(v) || v < 0.0) throw std::runtime_error("Invalid config value: " + item);
            if (key == "epsilon") {
                if (v >= 1.0) throw std::runtime_error("epsilon must be in [0, 1)");
                c.epsilon = v;
            } else if (key == "roulette") {
                if (v > 1.0) throw std::runtime_error("roulette must be in [0, 1]");
                c.roulette = v;
            } else if (key == "split") {
                if (v != 0.0 && v < 1.0) throw std::runtime_error("split must be 0 or at least 1");
                c.split = v;
            } else {
                c.cap = v;
            }
        } else if (key == "importance") c.importance = as_int(0, 1) != 0;
        else if (key == "graphs") c.graphs = as_int(0, 1) != 0;
        else if (key == "orders") c.orders = as_int(0, 1) != 0;
        else if (key == "rectangles") c.rectangles = as_int(0, 1) != 0;
        else if (key == "tail") c.tail = uint32_t(as_int(0, 1l << 26));
        else if (key == "fused") c.fused = int(as_int(-1, 1));
        else throw std::runtime_error("Unknown config key: " + key);
    }
    if (c.block % 32) throw std::runtime_error("block must be a multiple of 32");
    if (c.split > 0.0 && (c.roulette <= 0.0 || c.importance))
        throw std::runtime_error("splitting needs a roulette weight and no importance tally");
    if (!c.wavefront && (c.epsilon > 0.0 || c.roulette > 0.0 || c.importance || c.orders))
        throw std::runtime_error("guided transport, importance and scattering-order tallies need engine=wavefront");
    return c;
}

// Parsed transport table stream (transport.bin v1, kernels/cpu/worker.f90:1102-1120;
// version 2 adds one view azimuth per view after the view zeniths).
struct Prepared {
    int nx, ny, nz, nmat, angles, ntypes;
    bool paths, backward;
    double xunit, yunit, depol, vartheta0, phi0;
    std::vector<double> zunit, vartheta, vphi, albedo, beta, fractions, ssalb_gas;
    struct Lut { int n; double ssalb; std::vector<double> cos, cdf, f11, f22, f33, f12, f34, f44; };
    std::vector<Lut> luts;
};

inline Prepared parse(const double* raw, size_t count) {
    Prepared p{};
    size_t off = 0;
    auto take = [&](size_t n) {
        if (off + n > count) throw std::runtime_error("Truncated transport export");
        const double* q = raw + off;
        off += n;
        return q;
    };
    auto integer = [](double v) {
        if (!std::isfinite(v) || v != std::floor(v) || std::fabs(v) > 1e9)
            throw std::runtime_error("Unsupported transport export version or dimensions");
        return int(v);
    };
    if (!raw || count < 18) throw std::runtime_error("Invalid/nonfinite prepared transport export");
    for (size_t q = 0; q < count; ++q)
        if (!std::isfinite(raw[q])) throw std::runtime_error("Invalid/nonfinite prepared transport export");
    const double* h = take(12);
    int version = integer(h[0]);
    if (version < 1 || version > 3) throw std::runtime_error("Unsupported transport export version");
    p.nx = integer(h[1]); p.ny = integer(h[2]); p.nz = integer(h[3]);
    p.nmat = integer(h[4]); p.angles = integer(h[5]); p.ntypes = integer(h[6]);
    int ks = integer(h[7]), kd = integer(h[8]), kr = integer(h[9]);
    p.paths = integer(h[10]) != 0;
    p.backward = integer(h[11]) != 0;
    if (p.nx < 1 || p.ny < 1 || p.nz < 2 || p.nz > kMaxLayers || p.angles < 1 || p.angles > kMaxViews)
        throw std::runtime_error("Scene exceeds the supported grid limits");
    if (uint64_t(p.nx) * p.ny * p.nz > (1ull << 28) || p.nx > kMaxColumnsPerAxis || p.ny > kMaxColumnsPerAxis)
        throw std::runtime_error("Scene exceeds the supported grid limits");
    if ((p.nmat != 1 && p.nmat != 3 && p.nmat != 4) || p.ntypes < 0 || p.ntypes > kMaxSpecies ||
        ks != p.nz || kd != p.nz || kr != p.nz)
        throw std::runtime_error("CUDA supports I, IQU or IQUV, up to 3 particle species, TOA source/detector/grid");
    if (p.nmat == 4 && version < 3 && p.ntypes > 0)
        throw std::runtime_error("nmat 4 with particles needs the version 3 table stream (F34, F44)");
    const double* g = take(6);
    p.xunit = g[0]; p.yunit = g[1]; p.depol = g[2]; p.vartheta0 = g[3]; p.phi0 = g[4];
    const double phi = g[5];
    const size_t cols = size_t(p.nx) * p.ny, cells = cols * p.nz;
    const double* q = take(p.nz); p.zunit.assign(q, q + p.nz);
    q = take(p.angles); p.vartheta.assign(q, q + p.angles);
    if (version >= 2) { q = take(p.angles); p.vphi.assign(q, q + p.angles); }
    else p.vphi.assign(p.angles, phi);
    const double* surface = take(cols);
    q = take(cols); p.albedo.assign(q, q + cols);
    const double* elevation = take(cols);
    q = take(cells); p.beta.assign(q, q + cells);
    q = take(cells * (p.ntypes + 1)); p.fractions.assign(q, q + cells * (p.ntypes + 1));
    q = take(p.nz); p.ssalb_gas.assign(q, q + p.nz);
    for (int sp = 0; sp < p.ntypes; ++sp) {
        const double* hd = take(2);
        Prepared::Lut l;
        l.n = integer(hd[0]); l.ssalb = hd[1];
        if (l.n < 2 || l.n > 100000) throw std::runtime_error("Invalid scattering LUT size");
        const double* t = take(size_t(l.n) * 6);
        l.cos.assign(t, t + l.n); l.cdf.assign(t + l.n, t + 2 * l.n);
        l.f11.assign(t + 2 * l.n, t + 3 * l.n); l.f22.assign(t + 3 * l.n, t + 4 * l.n);
        l.f33.assign(t + 4 * l.n, t + 5 * l.n); l.f12.assign(t + 5 * l.n, t + 6 * l.n);
        if (version >= 3) {
            const double* v = take(size_t(l.n) * 2);
            l.f34.assign(v, v + l.n); l.f44.assign(v + l.n, v + 2 * l.n);
        }
        p.luts.push_back(std::move(l));
    }
    if (off != count) throw std::runtime_error("Trailing data in transport export");
    for (size_t c = 0; c < cols; ++c)
        if (surface[c] != -1 || elevation[c] != 1)
            throw std::runtime_error("CUDA supports only flat Lambertian surfaces");
    for (double z : p.zunit) if (!(z > 0)) throw std::runtime_error("Invalid layer dimensions, extinction, or scattering angle grid");
    for (double b : p.beta) if (b < 0) throw std::runtime_error("Invalid layer dimensions, extinction, or scattering angle grid");
    for (double v : p.vartheta) if (!(v >= 0 && v < 90)) throw std::runtime_error("Viewing zenith angles must be in [0, 90)");
    for (double a : p.albedo) if (!(a >= 0 && a <= 1)) throw std::runtime_error("Surface albedo must be in [0, 1]");
    for (const auto& l : p.luts) {
        for (int i = 1; i < l.n; ++i)
            if (!(l.cos[i] > l.cos[i - 1]) || l.cdf[i] < l.cdf[i - 1])
                throw std::runtime_error("Invalid layer dimensions, extinction, or scattering angle grid");
        if (std::fabs(l.cdf[0]) > 1e-12 || std::fabs(l.cdf[l.n - 1] - 1) > 1e-9)
            throw std::runtime_error("Invalid scattering CDF");
        // The bracket search guesses the index from a uniform 0..180 degree grid.
        for (int i = 0; i < l.n; ++i) {
            double angle = 180.0 - 180.0 * i / (l.n - 1);
            if (std::fabs(std::acos(std::max(-1.0, std::min(1.0, l.cos[i]))) / kDegToRad - angle) > 1e-6 * 180.0 + 1e-9)
                throw std::runtime_error("Scattering LUT must use a uniform angle grid from 180 to 0 degrees");
        }
    }
    return p;
}

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Mass kept by the analog particle sampler: the integral over the cosine of the proposal
// density (the bound CDF, linear between nodes) times F11 / (F11 + |F12|), four-point
// Gauss-Legendre per table interval; exactly the CDF span when F12 = 0 or nmat = 1.
inline double analog_norm(const Prepared::Lut& l, int nmat) {
    static const double xg[4] = {-0.8611363115940526, -0.3399810435848563, 0.3399810435848563, 0.8611363115940526};
    static const double wg[4] = {0.3478548451374538, 0.6521451548625461, 0.6521451548625461, 0.3478548451374538};
    double z = 0.0;
    for (int lo = 0; lo + 1 < l.n; ++lo) {
        const double dc = l.cdf[size_t(lo) + 1] - l.cdf[size_t(lo)];
        if (dc == 0.0) continue;
        if (nmat == 1 || (l.f12[size_t(lo)] == 0.0 && l.f12[size_t(lo) + 1] == 0.0)) { z += dc; continue; }
        double mean = 0.0;
        for (int q = 0; q < 4; ++q) {
            const double t = 0.5 * (xg[q] + 1.0);
            const double f11 = l.f11[size_t(lo)] + t * (l.f11[size_t(lo) + 1] - l.f11[size_t(lo)]);
            const double f12 = l.f12[size_t(lo)] + t * (l.f12[size_t(lo) + 1] - l.f12[size_t(lo)]);
            const double b = f11 + std::fabs(f12);
            mean += 0.5 * wg[q] * (b > 0.0 ? f11 / b : 0.0);
        }
        z += dc * mean;
    }
    return z;
}

// Host image of the device scene: element offsets into one allocation of T, plus the
// guide tables (int) appended after the T region.
template <typename T>
struct Packed {
    std::vector<T> values;
    std::vector<int> guides;
    size_t cells, zunit, zsum, ssalb_gas, albedo, tau_above, layer_beta, vprefix, run_lo, run_hi;
    size_t lut_f[kMaxSpecies], lut_cos[kMaxSpecies], lut_cdf[kMaxSpecies], guide[kMaxSpecies];
    size_t lut_v[kMaxSpecies];
    size_t band, band_count, extent;
    int uniform_top;
};

template <typename T>
Packed<T> pack(const Prepared& p, bool uniform_prefix, bool rectangles = true) {
    Packed<T> k{};
    auto& v = k.values;
    const size_t cols = size_t(p.nx) * p.ny, ncell = cols * p.nz;
    auto reserve = [&](size_t n) { size_t at = v.size(); v.resize(align_up(at + n, 4), T(0)); return at; };
    k.cells = reserve(4 * ncell);
    for (size_t c = 0; c < ncell; ++c) {
        v[k.cells + 4 * c] = T(p.beta[c]);
        double work = 0.0;  // cumulative fraction in the order of mc.f90:1028-1036
        for (int s = 0; s < p.ntypes; ++s) {
            work = s == 0 ? p.fractions[c * (p.ntypes + 1)] : work + p.fractions[c * (p.ntypes + 1) + s];
            v[k.cells + 4 * c + 1 + s] = T(work);
        }
        for (int s = p.ntypes; s < 3; ++s) v[k.cells + 4 * c + 1 + s] = T(2);  // never selected
    }
    k.zunit = reserve(p.nz);
    for (int z = 0; z < p.nz; ++z) v[k.zunit + z] = T(p.zunit[z]);
    k.zsum = reserve(p.nz + 1);
    {
        double acc = 0.0;
        v[k.zsum] = T(0);
        for (int z = 0; z < p.nz; ++z) { acc += p.zunit[z]; v[k.zsum + z + 1] = T(acc); }
    }
    k.ssalb_gas = reserve(p.nz);
    for (int z = 0; z < p.nz; ++z) v[k.ssalb_gas + z] = T(p.ssalb_gas[z]);
    k.albedo = reserve(cols);
    for (size_t c = 0; c < cols; ++c) v[k.albedo + c] = T(p.albedo[c]);
    // Highest horizontally varying physical layer, compared at transport precision.
    int varying = -1;
    for (int z = 0; z < p.nz - 1; ++z) {
        T b0 = T(p.beta[size_t(z) * cols]);
        for (size_t c = 1; c < cols; ++c)
            if (T(p.beta[size_t(z) * cols + c]) != b0) { varying = z; break; }
    }
    k.uniform_top = uniform_prefix ? varying + 1 : p.nz;
    // Extinction of the cells below the uniform top: the cell walks read nothing else.
    k.band_count = cols * size_t(std::min(k.uniform_top, p.nz - 1));
    k.band = reserve(k.band_count + 4);
    for (size_t c = 0; c < k.band_count; ++c) v[k.band + c] = T(p.beta[c]);
    // Equal-extinction rectangles of every band layer (greedy: from the first unassigned
    // cell in row order, widen along +x while the extinction is equal, then grow along +y
    // while the whole row segment is equal), stored per cell as its distances in cells to
    // the rectangle's faces, clamped to 255 (a clamped rectangle is still uniform).
    k.extent = SIZE_MAX;
    if (rectangles && k.band_count) {
        k.extent = k.guides.size();
        k.guides.resize(k.extent + k.band_count, 0);
        std::vector<char> taken(cols);
        for (size_t layer = 0; layer < k.band_count / cols; ++layer) {
            const T* b = v.data() + k.band + layer * cols;
            std::fill(taken.begin(), taken.end(), 0);
            for (int j0 = 0; j0 < p.ny; ++j0)
                for (int i0 = 0; i0 < p.nx; ++i0) {
                    const size_t c0 = size_t(i0) + size_t(p.nx) * j0;
                    if (taken[c0]) continue;
                    const T b0 = b[c0];
                    int i1 = i0;
                    while (i1 + 1 < p.nx && !taken[c0 + (i1 + 1 - i0)] && b[c0 + (i1 + 1 - i0)] == b0) ++i1;
                    int j1 = j0;
                    for (bool grow = true; grow && j1 + 1 < p.ny;) {
                        const size_t row = size_t(p.nx) * (j1 + 1);
                        for (int i = i0; i <= i1 && grow; ++i) grow = !taken[row + i] && b[row + i] == b0;
                        if (grow) ++j1;
                    }
                    for (int j = j0; j <= j1; ++j)
                        for (int i = i0; i <= i1; ++i) {
                            const size_t c = size_t(i) + size_t(p.nx) * j;
                            taken[c] = 1;
                            const uint32_t word = uint32_t(std::min(i - i0, 255)) | (uint32_t(std::min(i1 - i, 255)) << 8) |
                                                  (uint32_t(std::min(j - j0, 255)) << 16) | (uint32_t(std::min(j1 - j, 255)) << 24);
                            k.guides[k.extent + layer * cols + c] = int(word);
                        }
                }
        }
    }
    k.tau_above = reserve(p.nz);
    {
        // tau_above[k] = sum over physical layers above k of thickness * extinction,
        // accumulated from the top at transport precision.
        T acc = T(0);
        v[k.tau_above + p.nz - 1] = T(0);
        if (p.nz >= 2) v[k.tau_above + p.nz - 2] = T(0);
        for (int z = p.nz - 3; z >= 0; --z) {
            acc += T(p.zunit[z + 1]) * T(p.beta[size_t(z + 1) * cols]);
            v[k.tau_above + z] = acc;
        }
    }
    // Horizontally uniform layers (equal extinction in every cell at transport precision)
    // and the runs of consecutive uniform layers; the vacuum layer is uniform and clear.
    k.layer_beta = reserve(p.nz);
    k.vprefix = reserve(p.nz + 1);
    std::vector<bool> uniform(size_t(p.nz), true);
    for (int z = 0; z < p.nz - 1; ++z) {
        T b0 = T(p.beta[size_t(z) * cols]);
        for (size_t c = 1; c < cols && uniform[size_t(z)]; ++c)
            if (T(p.beta[size_t(z) * cols + c]) != b0) uniform[size_t(z)] = false;
        v[k.layer_beta + z] = uniform[size_t(z)] ? b0 : T(-1);
    }
    v[k.layer_beta + p.nz - 1] = T(0);
    {
        T acc = T(0);
        v[k.vprefix] = T(0);
        for (int z = 0; z < p.nz; ++z) {
            if (uniform[size_t(z)]) acc += T(v[k.layer_beta + z]) * T(p.zunit[size_t(z)]);
            v[k.vprefix + z + 1] = acc;
        }
    }
    k.run_lo = k.guides.size();
    for (int z = 0; z < p.nz; ++z) {
        int lo = z;
        while (uniform[size_t(z)] && lo > 0 && uniform[size_t(lo - 1)]) --lo;
        k.guides.push_back(lo);
    }
    k.run_hi = k.guides.size();
    for (int z = 0; z < p.nz; ++z) {
        int hi = z;
        while (uniform[size_t(z)] && hi < p.nz - 1 && uniform[size_t(hi + 1)]) ++hi;
        k.guides.push_back(hi);
    }
    for (int s = 0; s < p.ntypes; ++s) {
        const auto& l = p.luts[s];
        k.lut_f[s] = reserve(4 * size_t(l.n));
        for (int i = 0; i < l.n; ++i) {
            v[k.lut_f[s] + 4 * i] = T(l.f11[i]); v[k.lut_f[s] + 4 * i + 1] = T(l.f22[i]);
            v[k.lut_f[s] + 4 * i + 2] = T(l.f33[i]); v[k.lut_f[s] + 4 * i + 3] = T(l.f12[i]);
        }
        k.lut_cos[s] = reserve(l.n);
        for (int i = 0; i < l.n; ++i) v[k.lut_cos[s] + i] = T(l.cos[i]);
        k.lut_cdf[s] = reserve(l.n);
        for (int i = 0; i < l.n; ++i) v[k.lut_cdf[s] + i] = T(l.cdf[i]);
        k.lut_v[s] = SIZE_MAX;
        if (p.nmat == 4) {
            k.lut_v[s] = reserve(2 * size_t(l.n));
            for (int i = 0; i < l.n; ++i) {
                v[k.lut_v[s] + 2 * i] = T(l.f34[i]);
                v[k.lut_v[s] + 2 * i + 1] = T(l.f44[i]);
            }
        }
        // Guide: largest i <= n - 2 with cdf[i] <= g / kGuide (at transport precision).
        k.guide[s] = k.guides.size();
        int i = 0;
        for (int gidx = 0; gidx <= kGuide; ++gidx) {
            T level = T(gidx) / T(kGuide);
            while (i < l.n - 2 && T(l.cdf[i + 1]) <= level) ++i;
            k.guides.push_back(i);
        }
    }
    return k;
}

inline void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

template <typename T>
SceneView<T> make_view(const Prepared& p, const Packed<T>& k, void* base) {
    SceneView<T> s{};
    const T* tv = static_cast<const T*>(base);
    const int* gv = reinterpret_cast<const int*>(static_cast<const char*>(base) + k.values.size() * sizeof(T));
    s.nx = p.nx; s.ny = p.ny; s.nz = p.nz; s.nmat = p.nmat; s.angles = p.angles; s.ntypes = p.ntypes;
    s.paths = p.paths; s.uniform_top = k.uniform_top;
    s.backward = p.backward ? 1 : 0;
    s.xunit = T(p.xunit); s.yunit = T(p.yunit); s.depol = T(p.depol);
    s.xinv = T(1) / s.xunit; s.yinv = T(1) / s.yunit;
    const double th0 = kDegToRad * p.vartheta0, ph0 = kDegToRad * p.phi0;
    s.a0 = T(std::sin(th0) * std::cos(ph0)); s.b0 = T(std::sin(th0) * std::sin(ph0)); s.c0 = T(std::cos(th0));
    s.inv_mu0 = T(1) / std::fabs(s.c0);  // the flush's 1 / |mu0|, from the same rounded cosine
    s.phi0 = T(ph0);
    for (int ia = 0; ia < p.angles; ++ia) {
        double th = kDegToRad * p.vartheta[ia], ph = kDegToRad * p.vphi[ia];
        s.va[ia] = T(std::cos(ph) * std::sin(th)); s.vb[ia] = T(std::sin(ph) * std::sin(th));
        s.vc[ia] = T(std::cos(th)); s.vphi[ia] = T(ph);
        s.vsin[ia] = T(std::sqrt(std::max(1e-16, 1.0 - double(s.vc[ia]) * double(s.vc[ia]))));
        s.vcos_phi[ia] = T(std::cos(double(s.vphi[ia]))); s.vsin_phi[ia] = T(std::sin(double(s.vphi[ia])));
    }
    s.cells = tv + k.cells; s.zunit = tv + k.zunit; s.zsum = tv + k.zsum; s.ssalb_gas = tv + k.ssalb_gas;
    s.albedo = tv + k.albedo; s.tau_above = tv + k.tau_above;
    s.layer_beta = tv + k.layer_beta; s.vprefix = tv + k.vprefix;
    s.run_lo = gv + k.run_lo; s.run_hi = gv + k.run_hi;
    s.band = tv + k.band;
    const size_t band_bytes = align_up(k.band_count * sizeof(T), 16);
    s.band_bytes = (k.band_count && band_bytes <= kBandMaxBytes) ? uint32_t(band_bytes) : 0u;
    s.extent = k.extent == SIZE_MAX ? nullptr : reinterpret_cast<const uint32_t*>(gv + k.extent);
    for (int sp = 0; sp < p.ntypes; ++sp) {
        s.lut_n[sp] = p.luts[sp].n; s.ssalb_aer[sp] = T(p.luts[sp].ssalb);
        s.znorm[sp] = T(analog_norm(p.luts[sp], p.nmat));
        s.lut_f[sp] = tv + k.lut_f[sp]; s.lut_cos[sp] = tv + k.lut_cos[sp]; s.lut_cdf[sp] = tv + k.lut_cdf[sp];
        s.guide[sp] = gv + k.guide[sp];
        s.lut_v[sp] = k.lut_v[sp] == SIZE_MAX ? nullptr : tv + k.lut_v[sp];
    }
    return s;
}


}  // namespace host
}  // namespace monki
