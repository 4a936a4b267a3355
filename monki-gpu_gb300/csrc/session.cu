// C-ABI session for MONKI photon transport on one GB300 (sm_103a).
//
// The boundary mirrors the Metal bridge ABI v2 of the reference (kernels/metal/bridge.m:
// create :30-84, run :88-133, gpu_seconds :135, device_name :140, close :145) with the
// CUDA names declared in include/monki_cuda.h. A session owns: the packed scene, the FP32
// (or FP64) tally banks of one round group, the FP64 per-round output, a failure word and
// the work counters, all allocated once at create time (with the wavefront engine also the
// photon pool and its work lists). A run launches the transport kernels (wavefront
// iterations, captured as CUDA graphs, then the tail kernel; or the one-thread-per-history
// megakernel) and the FP64 flush on the session stream, copies the finished rounds to the
// caller's buffer and reports any failure flag as an error; it never falls back to the CPU.
#include <cuda_runtime.h>
#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <string>
#include <mutex>
#include <tuple>
#include <utility>
#include <vector>

#include "tail.h"
#include "statistics.cuh"
#include "wavefront.cuh"

namespace monki {
namespace {

constexpr double kDegToRad = 0.017453292519943295;

struct Config {
    bool fp64 = false;
    bool wavefront = true;       // engine=wavefront (default) or engine=megakernel
    uint32_t shards = 8;
    int block = 256;
    int blocks_per_sm = 0;       // 0 = occupancy-derived
    bool uniform_prefix = true;
    uint32_t pool = 1u << 20;    // wavefront photon slots
    uint32_t check_every = 8;    // wavefront iterations between host checks
    uint32_t walk = 24;          // walk steps per photon per transit launch
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

Config parse_config(const char* text) {
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

Prepared parse(const double* raw, size_t count) {
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
    if (uint64_t(p.nx) * p.ny * p.nz > (1ull << 28)) throw std::runtime_error("Scene exceeds the supported grid limits");
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

size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

// Mass kept by the analog particle sampler: the integral over the cosine of the proposal
// density (the bound CDF, linear between nodes) times F11 / (F11 + |F12|), four-point
// Gauss-Legendre per table interval; exactly the CDF span when F12 = 0 or nmat = 1.
double analog_norm(const Prepared::Lut& l, int nmat) {
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

struct Session {
    int device = 0;
    Config cfg;
    Prepared prep;
    cudaStream_t stream = nullptr;
    cudaEvent_t t0 = nullptr, t1 = nullptr, t2 = nullptr;
    void* scene = nullptr;        // T values then int guides
    void* banks = nullptr;        // round_capacity x shards x tally count, TA
    double* out = nullptr;        // round_capacity x tally count
    double* mu0mu = nullptr;
    uint32_t* failure = nullptr;
    unsigned long long* counters = nullptr;
    uint32_t* tail_next = nullptr;   // slot counter of the tail launch
    uint64_t tails = 0;              // tail launches so far
    uint32_t round_capacity = 1;
    TallyLayout layout{};       // output layout (and the megakernel's device layout)
    WaveTally wave{};           // wavefront device layout
    void* pool_memory = nullptr;
    Pool<float> pool32{};
    Pool<double> pool64{};
    double* flush_info = nullptr;
    void* scale = nullptr;            // per-cell roulette scale (T), or null
    double* importance = nullptr;     // 2 * cells, pilot runs only
    double* stats = nullptr;          // FP64 round statistics (statistics_layout), lazily
    double* history = nullptr;        // round_capacity x nmat spatial sums
    uint64_t stats_rounds = 0;
    void* pixel_weight = nullptr;     // nx * ny * angles (T), or null
    uint32_t* host_counts = nullptr;  // pinned
    uint64_t iterations = 0;
    // Per-stage event timing of the wavefront (runs with the profiling flag set):
    // 4 events per iteration of one host-check batch; ms summed per stage.
    std::vector<cudaEvent_t> stage_events;
    double stage_ms[3] = {0, 0, 0};
    uint64_t stage_launches[3] = {0, 0, 0};
    SceneView<float> view32{};
    SceneView<double> view64{};
    int grid = 0;
    double gpu_seconds = 0.0;
    // scatters, free-path cell visits, detector cell visits, tally updates, photons,
    // kernel launches
    uint64_t totals[6] = {0, 0, 0, 0, 0, 0};
    float last_kernel_ms = 0.f;   // transport kernel
    float last_run_ms = 0.f;      // transport kernel + FP64 flush
    std::string name;
};

void check(cudaError_t e, const char* what) {
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

template <typename T>
void upload(Session& s) {
    Packed<T> k = pack<T>(s.prep, s.cfg.uniform_prefix, s.cfg.rectangles);
    size_t bytes = k.values.size() * sizeof(T) + k.guides.size() * sizeof(int);
    check(cudaMalloc(&s.scene, std::max<size_t>(bytes, 16)), "cudaMalloc(scene)");
    // Stream-ordered copies, complete before the host image goes out of scope.
    check(cudaMemcpyAsync(s.scene, k.values.data(), k.values.size() * sizeof(T), cudaMemcpyHostToDevice, s.stream),
          "upload(scene)");
    if (!k.guides.empty())
        check(cudaMemcpyAsync(static_cast<char*>(s.scene) + k.values.size() * sizeof(T), k.guides.data(),
                              k.guides.size() * sizeof(int), cudaMemcpyHostToDevice, s.stream), "upload(guides)");
    check(cudaStreamSynchronize(s.stream), "upload");
    SceneView<T> v = make_view<T>(s.prep, k, s.scene);
    if constexpr (sizeof(T) == 4) s.view32 = v; else s.view64 = v;
}

template <typename T>
Pool<T> allocate_pool(Session& s) {
    const size_t n = s.cfg.pool;
    const size_t nz = size_t(s.prep.nz);
    const size_t quad = n * sizeof(Quad<T>);
    const size_t ring = s.cfg.importance ? n * kRing : 0;
    const size_t parts[] = {quad, quad, quad, n * sizeof(uint4), n * sizeof(uint32_t), n,
                            n * nz * sizeof(T), n * sizeof(uint32_t), 2 * n * sizeof(T),
                            10 * n * sizeof(uint32_t), kCountWords * sizeof(uint32_t),
                            ring * sizeof(uint32_t), ring * sizeof(T), s.cfg.importance ? n * sizeof(uint32_t) : 0,
                            s.cfg.orders ? n * sizeof(uint32_t) : 0,
                            (s.prep.nmat == 4 && !s.prep.backward) ? n * sizeof(T) : 0,
                            s.prep.backward ? size_t(s.prep.nmat) * s.prep.nmat * n * sizeof(T) : 0,
                            (s.prep.backward && s.cfg.orders) ? n * sizeof(uint32_t) : 0,
                            s.cfg.split > 0.0 ? n * sizeof(uint32_t) : 0,
                            s.cfg.split > 0.0 ? n * kSplitStack * sizeof(SplitCopy<T>) : 0,
                            s.cfg.split > 0.0 ? n * sizeof(uint32_t) : 0};
    size_t bytes = 0;
    for (size_t part : parts) bytes += align_up(part, 256);
    check(cudaMalloc(&s.pool_memory, bytes), "cudaMalloc(pool)");
    char* p = static_cast<char*>(s.pool_memory);
    auto take = [&](size_t b) { char* q = p; p += align_up(b, 256); return q; };
    Pool<T> P{};
    P.capacity = uint32_t(n);
    P.pos = reinterpret_cast<Quad<T>*>(take(quad));
    P.dir = reinterpret_cast<Quad<T>*>(take(quad));
    P.pol = reinterpret_cast<Quad<T>*>(take(quad));
    P.meta = reinterpret_cast<uint4*>(take(n * sizeof(uint4)));
    P.steps = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
    P.kind = reinterpret_cast<uint8_t*>(take(n));
    P.wander = reinterpret_cast<T*>(take(n * nz * sizeof(T)));
    P.runs = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
    P.run_ci = reinterpret_cast<T*>(take(2 * n * sizeof(T)));
    uint32_t* lists = reinterpret_cast<uint32_t*>(take(10 * n * sizeof(uint32_t)));
    for (int b = 0; b < 2; ++b) {
        for (int q = 0; q < 3; ++q) P.queue[b][q] = lists + size_t(5 * b + q) * n;
        P.paused[b] = lists + size_t(5 * b + 3) * n;
        P.vacant[b] = lists + size_t(5 * b + 4) * n;
    }
    P.counts = reinterpret_cast<uint32_t*>(take(kCountWords * sizeof(uint32_t)));
    if (s.cfg.importance) {
        P.ring_cell = reinterpret_cast<uint32_t*>(take(ring * sizeof(uint32_t)));
        P.ring_inv = reinterpret_cast<T*>(take(ring * sizeof(T)));
        P.ring_n = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
        P.importance = s.importance;
    }
    if (s.cfg.orders) P.order = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
    if (s.prep.nmat == 4 && !s.prep.backward) P.vee = reinterpret_cast<T*>(take(n * sizeof(T)));
    if (s.prep.backward) P.matrix = reinterpret_cast<T*>(take(size_t(s.prep.nmat) * s.prep.nmat * n * sizeof(T)));
    if (s.prep.backward && s.cfg.orders) P.first = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
    if (s.cfg.split > 0.0) {
        P.lineage = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
        P.copies = reinterpret_cast<SplitCopy<T>*>(take(n * kSplitStack * sizeof(SplitCopy<T>)));
        P.waiting = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
    }
    return P;
}

template <typename T, int NMAT, bool PATHS>
const void* kernel_symbol() { return reinterpret_cast<const void*>(&transport_kernel<T, T, NMAT, PATHS>); }

template <typename T>
void launch_transport(Session& s, const Controls& c, int grid) {
    const SceneView<T>& v = [&]() -> const SceneView<T>& {
        if constexpr (sizeof(T) == 4) return s.view32; else return s.view64;
    }();
    T* banks = static_cast<T*>(s.banks);
    const int nm = s.prep.nmat;
    const bool paths = s.prep.paths;
    if (nm == 1 && !paths) transport_kernel<T, T, 1, false><<<grid, s.cfg.block, 0, s.stream>>>(v, c, banks, s.layout, s.failure, s.counters);
    else if (nm == 1) transport_kernel<T, T, 1, true><<<grid, s.cfg.block, 0, s.stream>>>(v, c, banks, s.layout, s.failure, s.counters);
    else if (!paths) transport_kernel<T, T, 3, false><<<grid, s.cfg.block, 0, s.stream>>>(v, c, banks, s.layout, s.failure, s.counters);
    else transport_kernel<T, T, 3, true><<<grid, s.cfg.block, 0, s.stream>>>(v, c, banks, s.layout, s.failure, s.counters);
}

// Stream work of a wavefront batch, either launched on the session stream at once or, with
// a graph, appended as a chain of graph nodes (kernel, memset and copy nodes built through
// the graph API). Building the graph node by node rather than by stream capture keeps it
// independent of what other host threads do meanwhile: a capture is invalidated by any
// device-wide synchronization (cudaFree, cudaDeviceSynchronize, a synchronous copy) that
// another session's thread makes while it is open.
struct Recorder {
    cudaStream_t stream = nullptr;
    cudaGraph_t graph = nullptr;     // null: launch on the stream
    cudaGraphNode_t last = nullptr;  // the chain's last node

    template <typename... P, typename... A>
    void kernel(void (*fn)(P...), unsigned grid, unsigned block, size_t smem, const A&... args) {
        static_assert(sizeof...(P) == sizeof...(A), "one argument per kernel parameter");
        std::tuple<P...> values(static_cast<P>(args)...);
        launch(reinterpret_cast<const void*>(fn), grid, block, smem, values, std::index_sequence_for<P...>{});
    }

    // count 32-bit words at dst set to zero.
    void clear(uint32_t* dst, size_t count) {
        if (!graph) {
            check(cudaMemsetAsync(dst, 0, count * sizeof(uint32_t), stream), "memset(lists)");
            return;
        }
        cudaMemsetParams m{};
        m.dst = dst;
        m.value = 0u;
        m.elementSize = sizeof(uint32_t);
        m.width = count;
        m.height = 1;
        cudaGraphNode_t node = nullptr;
        check(cudaGraphAddMemsetNode(&node, graph, last ? &last : nullptr, last ? 1 : 0, &m), "graph memset node");
        last = node;
    }

    void copy_to_host(void* dst, const void* src, size_t bytes) {
        if (!graph) {
            check(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, stream), "copy(counts)");
            return;
        }
        cudaGraphNode_t node = nullptr;
        check(cudaGraphAddMemcpyNode1D(&node, graph, last ? &last : nullptr, last ? 1 : 0, dst, src, bytes,
                                       cudaMemcpyDeviceToHost), "graph copy node");
        last = node;
    }

    // Per-stage timing events: stream launches only.
    void event(cudaEvent_t e) {
        if (e && !graph) check(cudaEventRecord(e, stream), "event");
    }

  private:
    template <typename Tuple, size_t... I>
    void launch(const void* fn, unsigned grid, unsigned block, size_t smem, Tuple& values, std::index_sequence<I...>) {
        void* params[] = {static_cast<void*>(&std::get<I>(values))...};
        if (!graph) {
            check(cudaLaunchKernel(fn, dim3(grid), dim3(block), params, smem, stream), "wavefront launch");
            return;
        }
        cudaKernelNodeParams p{};
        p.func = const_cast<void*>(fn);
        p.gridDim = dim3(grid);
        p.blockDim = dim3(block);
        p.sharedMemBytes = unsigned(smem);
        p.kernelParams = params;
        p.extra = nullptr;
        cudaGraphNode_t node = nullptr;
        check(cudaGraphAddKernelNode(&node, graph, last ? &last : nullptr, last ? 1 : 0, &p), "graph kernel node");
        last = node;
    }
};

template <typename T, int NMAT, bool PATHS>
void wave_iteration(Session& s, Recorder& rec, const SceneView<T>& v, Pool<T>& P, const Controls& c,
                    const Divisors& dv, int grid, uint32_t cur, cudaEvent_t* ev) {
    T* banks = static_cast<T*>(s.banks);
    const uint32_t out = cur ^ 1u;
    rec.clear(P.counts + kListCounts * out, kListCounts);
    if (ev) rec.event(ev[0]);
    // One thread per work-list entry (at most one per slot): a thread that looped over
    // several entries drifted away from its warp's other lanes (each walk has its own
    // length). The peel keeps the persistent grid, which measured faster.
    const unsigned slots_grid = (P.capacity + uint32_t(s.cfg.block) - 1) / uint32_t(s.cfg.block);
    const unsigned block = unsigned(s.cfg.block);
    Guide<T> g{T(s.cfg.epsilon), T(s.cfg.roulette), s.cfg.cap > 0.0 ? T(s.cfg.cap) : T(INFINITY),
               static_cast<const T*>(s.scale), T(s.cfg.split)};
    // Fused: each event's scattering and its photon's next walk in one kernel (the events of
    // the previous iteration, peeled there). Unfused (scenes with layer paths by default):
    // the walks in slot order, the peel-off, then the scatterings.
    const bool fused = s.cfg.fused == 1 || (s.cfg.fused < 0 && !PATHS);
    if (fused) {
        if (v.backward)
            rec.kernel(&wf_step<T, NMAT, PATHS, true>, slots_grid, block, v.band_bytes, v, c, dv, P, g, s.cfg.walk, cur,
                       s.failure, s.counters);
        else
            rec.kernel(&wf_step<T, NMAT, PATHS, false>, slots_grid, block, v.band_bytes, v, c, dv, P, g, s.cfg.walk, cur,
                       s.failure, s.counters);
    } else {
        rec.kernel(&wf_transit<T, PATHS>, slots_grid, block, v.band_bytes, v, c, dv, P, s.cfg.walk, out, s.failure,
                   s.counters);
    }
    if (ev) rec.event(ev[1]);
    if (v.backward)
        rec.kernel(&wf_peel<T, T, NMAT, PATHS, true>, unsigned(grid), block, v.band_bytes, v, c, dv, P, banks, s.wave,
                   out, s.failure, s.counters);
    else
        rec.kernel(&wf_peel<T, T, NMAT, PATHS, false>, unsigned(grid), block, v.band_bytes, v, c, dv, P, banks, s.wave,
                   out, s.failure, s.counters);
    if (ev) rec.event(ev[2]);
    if (!fused) {
        if (v.backward) rec.kernel(&wf_scatter<T, NMAT, true>, slots_grid, block, 0, v, c, dv, P, g, out, s.failure);
        else rec.kernel(&wf_scatter<T, NMAT, false>, slots_grid, block, 0, v, c, dv, P, g, out, s.failure);
    }
    if (ev) rec.event(ev[3]);
}

template <typename T>
void run_wavefront(Session& s, const Controls& c) {
    const SceneView<T>& v = [&]() -> const SceneView<T>& {
        if constexpr (sizeof(T) == 4) return s.view32; else return s.view64;
    }();
    Pool<T> P = [&]() -> Pool<T>& {
        if constexpr (sizeof(T) == 4) return s.pool32; else return s.pool64;
    }();
    P.pixel_weight = static_cast<const T*>(s.pixel_weight);
    // Small groups scan only as many slots as they have photons.
    P.capacity = uint32_t(std::min<uint64_t>(P.capacity, (uint64_t(c.count) + 255) / 256 * 256));
    wf_reset<T><<<int((P.capacity + 255) / 256), 256, 0, s.stream>>>(P);
    check(cudaGetLastError(), "reset launch");
    Divisors dv{FastDiv::make(c.per_round), FastDiv::make(uint32_t(s.prep.nx)), FastDiv::make(uint32_t(s.prep.ny)),
                FastDiv::make(uint32_t(s.prep.nx * s.prep.ny))};
    const int grid = s.grid;
    const int nm = s.prep.nmat;
    const bool paths = s.prep.paths;
    const uint64_t limit = uint64_t(c.max_steps) + 16;  // events per photon are bounded by its steps
    uint64_t it = 0, launches = 0;
    const bool profile = c.profile != 0;
    if (profile && s.stage_events.size() < 4 * size_t(s.cfg.check_every)) {
        for (cudaEvent_t e : s.stage_events) cudaEventDestroy(e);
        s.stage_events.assign(4 * size_t(s.cfg.check_every), nullptr);
        for (cudaEvent_t& e : s.stage_events) check(cudaEventCreate(&e), "cudaEventCreate");
    }
    if (profile) for (int q = 0; q < 3; ++q) { s.stage_ms[q] = 0; s.stage_launches[q] = 0; }
    // A batch is an even number of iterations, so each starts reading the work lists of
    // buffer 0 and leaves its last lists there.
    auto batch = [&](Recorder& rec) {
        for (uint32_t b = 0; b < s.cfg.check_every; ++b) {
            cudaEvent_t* ev = profile ? s.stage_events.data() + 4 * b : nullptr;
            const uint32_t cur = b & 1u;
            if (nm == 1 && !paths) wave_iteration<T, 1, false>(s, rec, v, P, c, dv, grid, cur, ev);
            else if (nm == 1) wave_iteration<T, 1, true>(s, rec, v, P, c, dv, grid, cur, ev);
            else if (nm == 4 && !paths) wave_iteration<T, 4, false>(s, rec, v, P, c, dv, grid, cur, ev);
            else if (nm == 4) wave_iteration<T, 4, true>(s, rec, v, P, c, dv, grid, cur, ev);
            else if (!paths) wave_iteration<T, 3, false>(s, rec, v, P, c, dv, grid, cur, ev);
            else wave_iteration<T, 3, true>(s, rec, v, P, c, dv, grid, cur, ev);
        }
        rec.copy_to_host(s.host_counts, P.counts, kCountWords * sizeof(uint32_t));
    };
    // Without per-stage timing, the batch of check_every iterations (2 launches and a list
    // reset each, then the counts read-back) is built once per run as a CUDA graph and
    // replayed: the host submits one launch per batch instead of 3 * check_every.
    struct GraphGuard {
        cudaGraph_t g = nullptr; cudaGraphExec_t e = nullptr;
        ~GraphGuard() { if (e) cudaGraphExecDestroy(e); if (g) cudaGraphDestroy(g); }
    } guard;
    Recorder direct{s.stream};
    if (s.cfg.graphs && !profile) {
        check(cudaGraphCreate(&guard.g, 0), "graph create");
        Recorder chain{s.stream, guard.g};
        batch(chain);
        check(cudaGraphInstantiate(&guard.e, guard.g, 0), "graph instantiate");
    }
    const cudaGraphExec_t exec = guard.e;
    for (;;) {
        if (exec) check(cudaGraphLaunch(exec, s.stream), "graph launch");
        else batch(direct);
        it += s.cfg.check_every;
        const bool fused = s.cfg.fused == 1 || (s.cfg.fused < 0 && !paths);
        launches += (fused ? 2 : 3) * uint64_t(s.cfg.check_every);
        check(cudaGetLastError(), "wavefront launch");
        check(cudaStreamSynchronize(s.stream), "wavefront");
        if (profile) {
            for (uint32_t b = 0; b < s.cfg.check_every; ++b) {
                for (int q = 0; q < 3; ++q) {
                    float ms = 0.f;
                    check(cudaEventElapsedTime(&ms, s.stage_events[4 * b + q], s.stage_events[4 * b + q + 1]), "stage time");
                    s.stage_ms[q] += ms;
                    s.stage_launches[q] += 1;
                }
            }
        }
        const uint32_t* h = s.host_counts;
        // Done when every photon was claimed and no slot is listed: no event waits for its
        // scattering, no walk is paused by the per-launch step budget, no vacant slot holds
        // split copies.
        const bool claimed = h[kClaimCount] >= c.count;
        const uint64_t live = uint64_t(h[0]) + h[1] + h[2] + h[3] + h[4];
        if (claimed && live == 0) break;
        // Few photons left and none to claim: run each to its end in one launch (not while
        // timing stages, which keeps the kernels apart).
        if (!profile && s.cfg.tail && claimed && live <= s.cfg.tail) {
            Guide<T> g{T(s.cfg.epsilon), T(s.cfg.roulette), s.cfg.cap > 0.0 ? T(s.cfg.cap) : T(INFINITY),
                       static_cast<const T*>(s.scale), T(s.cfg.split)};
            check(launch_tail<T>(v, c, dv, P, static_cast<T*>(s.banks), s.wave, g, 0u, fused, s.failure, s.counters,
                                 s.tail_next, s.stream), "tail launch");
            check(cudaStreamSynchronize(s.stream), "tail");
            s.tails += 1;
            launches += 1;
            break;  // every photon of the group has ended
        }
        if (it > limit * 4 + 1024 && it > 1000000) throw std::runtime_error("wavefront did not drain");
    }
    s.iterations += it;
    s.totals[5] += launches;
}

template <typename T>
int occupancy(const Session& s) {
    const void* fn;
    if (s.prep.nmat == 1) fn = s.prep.paths ? kernel_symbol<T, 1, true>() : kernel_symbol<T, 1, false>();
    else fn = s.prep.paths ? kernel_symbol<T, 3, true>() : kernel_symbol<T, 3, false>();
    int blocks = 0;
    check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, s.cfg.block, 0), "occupancy");
    return std::max(blocks, 1);
}

void destroy(Session* s) {
    if (!s) return;
    cudaSetDevice(s->device);
    if (s->stream) cudaStreamSynchronize(s->stream);
    cudaFree(s->scene); cudaFree(s->banks); cudaFree(s->out); cudaFree(s->mu0mu);
    cudaFree(s->failure); cudaFree(s->counters); cudaFree(s->tail_next);
    cudaFree(s->pool_memory); cudaFree(s->flush_info); cudaFree(s->scale); cudaFree(s->importance); cudaFree(s->pixel_weight);
    cudaFree(s->stats); cudaFree(s->history);
    if (s->host_counts) cudaFreeHost(s->host_counts);
    if (s->t0) cudaEventDestroy(s->t0);
    if (s->t1) cudaEventDestroy(s->t1);
    if (s->t2) cudaEventDestroy(s->t2);
    for (cudaEvent_t e : s->stage_events) cudaEventDestroy(e);
    if (s->stream) cudaStreamDestroy(s->stream);
    delete s;
}

Controls group_controls(const Session& s, const uint32_t controls[8]) {
    Controls c{controls[0], controls[1], controls[2], controls[3], controls[4], controls[5], controls[6], controls[7]};
    if (!c.per_round || !c.rounds || c.rounds > s.round_capacity || !c.max_steps ||
        uint64_t(c.first) + c.count > uint64_t(c.per_round) * c.rounds)
        throw std::runtime_error("Invalid CUDA round group");
    return c;
}

// Transport and FP64 flush of one round group into s.out, on the session stream.
void execute(Session& s, const Controls& c) {
    check(cudaSetDevice(s.device), "cudaSetDevice");
    check(cudaMemsetAsync(s.failure, 0, sizeof(uint32_t), s.stream), "memset(failure)");
    check(cudaMemsetAsync(s.counters, 0, 4 * sizeof(unsigned long long), s.stream), "memset(counters)");
    const int needed = int(std::min<uint64_t>((uint64_t(c.count) + s.cfg.block - 1) / s.cfg.block, uint64_t(s.grid)));
    check(cudaEventRecord(s.t0, s.stream), "event");
    if (c.count) {
        if (s.cfg.wavefront) {
            if (s.cfg.fp64) run_wavefront<double>(s, c); else run_wavefront<float>(s, c);
        } else {
            if (s.cfg.fp64) launch_transport<double>(s, c, std::max(needed, 1));
            else launch_transport<float>(s, c, std::max(needed, 1));
            s.totals[5] += 1;
        }
        check(cudaGetLastError(), "transport launch");
    }
    check(cudaEventRecord(s.t1, s.stream), "event");
    const uint64_t total = uint64_t(s.layout.count) * c.rounds;
    const int fgrid = int(std::min<uint64_t>((total + 255) / 256, 4096));
    const Prepared& p = s.prep;
    if (s.cfg.wavefront) {
        if (s.cfg.fp64)
            wf_flush<double><<<fgrid, 256, 0, s.stream>>>(static_cast<const double*>(s.banks), s.wave, p.nmat,
                p.nx, p.ny, p.nz, p.angles, s.flush_info, c.rounds, s.layout.count, p.paths, s.out);
        else
            wf_flush<float><<<fgrid, 256, 0, s.stream>>>(static_cast<const float*>(s.banks), s.wave, p.nmat,
                p.nx, p.ny, p.nz, p.angles, s.flush_info, c.rounds, s.layout.count, p.paths, s.out);
        check(cudaGetLastError(), "flush launch");
        const size_t elem = s.cfg.fp64 ? sizeof(double) : sizeof(float);
        check(cudaMemsetAsync(s.banks, 0, size_t(c.rounds) * s.wave.shards * s.wave.count * elem, s.stream),
              "memset(banks)");
    } else {
        if (s.cfg.fp64)
            flush_kernel<double><<<fgrid, 256, 0, s.stream>>>(static_cast<double*>(s.banks), s.layout, p.nmat,
                p.nx, p.ny, p.nz, p.angles, s.mu0mu, c.rounds, s.out);
        else
            flush_kernel<float><<<fgrid, 256, 0, s.stream>>>(static_cast<float*>(s.banks), s.layout, p.nmat,
                p.nx, p.ny, p.nz, p.angles, s.mu0mu, c.rounds, s.out);
        check(cudaGetLastError(), "flush launch");
    }
    check(cudaEventRecord(s.t2, s.stream), "event");
    s.totals[5] += 1;  // the flush
}

// Wait for the group, collect timing and counters, and turn a failure flag into an error.
void finish(Session& s, const Controls& c) {
    uint32_t flag = 0;
    unsigned long long cnt[4] = {0, 0, 0, 0};
    check(cudaMemcpyAsync(&flag, s.failure, sizeof(flag), cudaMemcpyDeviceToHost, s.stream), "copy(failure)");
    check(cudaMemcpyAsync(cnt, s.counters, sizeof(cnt), cudaMemcpyDeviceToHost, s.stream), "copy(counters)");
    check(cudaStreamSynchronize(s.stream), "transport");
    float ms = 0.f, run_ms = 0.f;
    check(cudaEventElapsedTime(&ms, s.t0, s.t1), "elapsed");
    check(cudaEventElapsedTime(&run_ms, s.t0, s.t2), "elapsed");
    s.last_kernel_ms = ms;
    s.last_run_ms = run_ms;
    if (c.profile) s.gpu_seconds += run_ms * 1e-3;
    for (int q = 0; q < 4; ++q) s.totals[q] += cnt[q];
    s.totals[4] += c.count;
    if (flag) {
        char msg[128];
        std::snprintf(msg, sizeof msg, "CUDA transport failed (flag %u); round rejected", flag);
        throw std::runtime_error(msg);
    }
}

StatsLayout statistics_layout(const Session& s) {
    const Prepared& p = s.prep;
    const uint32_t pixels = uint32_t(p.nx) * uint32_t(p.ny) * uint32_t(p.angles);
    StatsLayout L{};
    L.stokes = uint32_t(p.nmat) * pixels;
    L.paths = p.paths ? pixels * uint32_t(p.nz) : 0u;
    L.weights = p.paths ? pixels : 0u;
    L.nz = uint32_t(p.nz);
    L.nx = uint32_t(p.nx);
    L.ny = uint32_t(p.ny);
    L.count = 3 * size_t(L.stokes) + 4 * size_t(L.paths) + 3 * size_t(L.weights);
    return L;
}

// Add the rounds of s.out to the device accumulators (FP64, rounds in order) and write the
// per-round spatial sums of the normalized Stokes tallies to the host.
void accumulate(Session& s, uint32_t rounds, double photons_per_column, double* history) {
    const StatsLayout L = statistics_layout(s);
    if (!s.stats) {
        check(cudaMalloc(&s.stats, L.count * sizeof(double)), "cudaMalloc(statistics)");
        check(cudaMemsetAsync(s.stats, 0, L.count * sizeof(double), s.stream), "memset(statistics)");
        check(cudaMalloc(&s.history, size_t(s.round_capacity) * s.prep.nmat * sizeof(double)), "cudaMalloc(history)");
    }
    const uint32_t elements = L.stokes + L.paths + L.weights;
    const int grid = int(std::min<uint32_t>((elements + 255) / 256, 8192));
    // Paths read the weight means of the previous groups, so the weights update second.
    stats_update<<<grid, 256, 0, s.stream>>>(s.out, uint32_t(s.layout.count), rounds, uint32_t(s.stats_rounds), L,
                                            photons_per_column, s.stats, 0);
    if (L.weights)
        stats_update<<<grid, 256, 0, s.stream>>>(s.out, uint32_t(s.layout.count), rounds, uint32_t(s.stats_rounds), L,
                                                photons_per_column, s.stats, 1);
    round_sums<<<dim3(rounds, uint32_t(s.prep.nmat)), 256, 0, s.stream>>>(s.out, uint32_t(s.layout.count),
                                                                          uint32_t(s.prep.nmat), L.stokes,
                                                                          photons_per_column, s.history);
    check(cudaGetLastError(), "statistics launch");
    check(cudaMemcpyAsync(history, s.history, size_t(rounds) * s.prep.nmat * sizeof(double), cudaMemcpyDeviceToHost,
                          s.stream), "copy(history)");
    check(cudaStreamSynchronize(s.stream), "statistics");
    s.stats_rounds += rounds;
}

void write_error(char* err, size_t n, const std::string& msg) {
    if (err && n) std::snprintf(err, n, "%s", msg.c_str());
}

}  // namespace
}  // namespace monki

using namespace monki;

extern "C" {

int monki_cuda_abi_version(void) { return 1; }

void* monki_cuda_create(uint32_t device, const double* tables, size_t table_count, uint32_t round_capacity,
                        const char* config, char* err, size_t errlen) {
    Session* s = nullptr;
    try {
        Config cfg = parse_config(config);
        Prepared prep = parse(tables, table_count);
        if ((prep.backward || prep.nmat == 4) && !cfg.wavefront)
            throw std::runtime_error("backward transport and nmat 4 need engine=wavefront");
        if (prep.backward && (cfg.epsilon > 0.0 || cfg.roulette > 0.0 || cfg.importance))
            throw std::runtime_error("guided transport and importance tallies need forward transport");
        if (cfg.split > 0.0 && prep.paths) throw std::runtime_error("splitting needs a scene without layer paths");
        if (round_capacity < 1 || round_capacity > 4096) throw std::runtime_error("round_capacity must be in [1, 4096]");
        int n = 0;
        cudaError_t e = cudaGetDeviceCount(&n);
        if (e != cudaSuccess || n == 0) throw std::runtime_error("No CUDA device is available");
        if (device >= uint32_t(n)) throw std::runtime_error("Requested CUDA device is unavailable");
        s = new Session();
        s->device = int(device);
        s->cfg = cfg;
        s->prep = std::move(prep);
        s->round_capacity = round_capacity;
        check(cudaSetDevice(s->device), "cudaSetDevice");
        cudaDeviceProp prop{};
        check(cudaGetDeviceProperties(&prop, s->device), "cudaGetDeviceProperties");
        if (prop.major < 10) throw std::runtime_error("This build targets sm_103a (GB300)");
        s->name = prop.name;
        check(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking), "cudaStreamCreate");
        check(cudaEventCreate(&s->t0), "cudaEventCreate");
        check(cudaEventCreate(&s->t1), "cudaEventCreate");
        check(cudaEventCreate(&s->t2), "cudaEventCreate");
        const Prepared& p = s->prep;
        TallyLayout& L = s->layout;
        L.stokes = uint32_t(p.nmat * p.nx * p.ny * p.angles);
        L.paths = p.paths ? uint32_t(p.nx * p.ny * p.nz * p.angles) : 0u;
        L.weights = p.paths ? uint32_t(p.nx * p.ny * p.angles) : 0u;
        L.orders = cfg.orders ? L.stokes + 2u * uint32_t(p.nmat * p.nx * p.ny * p.nz * p.angles) : 0u;
        L.count = L.stokes + L.paths + L.weights + L.orders;
        L.shards = cfg.shards;
        const uint32_t pixels = uint32_t(p.nx * p.ny * p.angles);
        WaveTally& W = s->wave;
        W.pixels = pixels;
        W.layers = p.paths ? pixels * uint32_t(p.nz + 1) * 4u : 0u;
        W.count = 4u * pixels + W.layers;
        W.locations = uint32_t(p.nx * p.ny * p.nz * p.angles);
        W.orders = cfg.orders ? W.count : 0u;
        if (cfg.orders) W.count += 4u * (pixels + 2u * W.locations);
        W.vee = p.nmat == 4 ? W.count : 0u;
        if (p.nmat == 4) W.count += pixels;
        W.shards = cfg.shards;
        const size_t elem = cfg.fp64 ? sizeof(double) : sizeof(float);
        const size_t per_round = cfg.wavefront ? W.count : L.count;
        const size_t bank_bytes = size_t(round_capacity) * L.shards * per_round * elem;
        check(cudaMalloc(&s->banks, bank_bytes), "cudaMalloc(banks)");
        check(cudaMemsetAsync(s->banks, 0, bank_bytes, s->stream), "cudaMemset(banks)");
        check(cudaMalloc(&s->out, size_t(round_capacity) * L.count * sizeof(double)), "cudaMalloc(out)");
        std::vector<double> mu(size_t(p.angles));
        // mu0/mu on forward Stokes tallies only (mc.f90:1456-1474).
        for (int ia = 0; ia < p.angles; ++ia)
            mu[size_t(ia)] = p.backward ? 1.0
                                        : std::fabs(std::cos(kDegToRad * p.vartheta0)) / std::fabs(std::cos(kDegToRad * p.vartheta[ia]));
        check(cudaMalloc(&s->mu0mu, mu.size() * sizeof(double)), "cudaMalloc(mu0mu)");
        check(cudaMemcpyAsync(s->mu0mu, mu.data(), mu.size() * sizeof(double), cudaMemcpyHostToDevice, s->stream),
              "upload(mu0mu)");
        check(cudaStreamSynchronize(s->stream), "upload(mu0mu)");
        check(cudaMalloc(&s->failure, sizeof(uint32_t)), "cudaMalloc(failure)");
        check(cudaMalloc(&s->tail_next, sizeof(uint32_t)), "cudaMalloc(tail)");
        check(cudaMalloc(&s->counters, 4 * sizeof(unsigned long long)), "cudaMalloc(counters)");
        if (cfg.fp64) upload<double>(*s); else upload<float>(*s);
        if (cfg.importance) {
            const size_t cells = size_t(p.nx) * p.ny * p.nz;
            check(cudaMalloc(&s->importance, 2 * cells * sizeof(double)), "cudaMalloc(importance)");
            check(cudaMemsetAsync(s->importance, 0, 2 * cells * sizeof(double), s->stream), "cudaMemset(importance)");
        }
        if (cfg.wavefront) {
            if (cfg.fp64) s->pool64 = allocate_pool<double>(*s); else s->pool32 = allocate_pool<float>(*s);
            std::vector<double> info(size_t(p.nz) + 1 + 2 * size_t(p.angles));
            for (int z = 0; z < p.nz; ++z) info[size_t(z)] = p.zunit[size_t(z)];
            // The same direction cosines the kernels use, rounded to transport precision.
            const double c0 = std::cos(kDegToRad * p.vartheta0);
            info[size_t(p.nz)] = 1.0 / std::fabs(cfg.fp64 ? c0 : double(float(c0)));
            for (int ia = 0; ia < p.angles; ++ia) {
                const double vc = std::cos(kDegToRad * p.vartheta[size_t(ia)]);
                info[size_t(p.nz) + 1 + ia] = 1.0 / std::fabs(cfg.fp64 ? vc : double(float(vc)));
                info[size_t(p.nz) + 1 + p.angles + ia] = mu[size_t(ia)];
            }
            check(cudaMalloc(&s->flush_info, info.size() * sizeof(double)), "cudaMalloc(flush info)");
            check(cudaMemcpyAsync(s->flush_info, info.data(), info.size() * sizeof(double), cudaMemcpyHostToDevice,
                                  s->stream), "upload(flush info)");
            check(cudaStreamSynchronize(s->stream), "upload(flush info)");
            check(cudaMallocHost(&s->host_counts, kCountWords * sizeof(uint32_t)), "cudaMallocHost(counts)");
        }
        int per_sm = cfg.blocks_per_sm;
        if (!per_sm) {
            if (cfg.wavefront) {
                int blocks = 0;
                const void* fn = cfg.fp64 ? reinterpret_cast<const void*>(&wf_peel<double, double, 3, true, false>)
                                          : reinterpret_cast<const void*>(&wf_peel<float, float, 3, true, false>);
                check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&blocks, fn, cfg.block, 0), "occupancy");
                per_sm = std::max(blocks, 1);
            } else {
                per_sm = cfg.fp64 ? occupancy<double>(*s) : occupancy<float>(*s);
            }
        }
        s->grid = prop.multiProcessorCount * per_sm;
        // This session's stream only: a device-wide synchronization would also wait for
        // (and stall) the sessions other host threads are running.
        check(cudaStreamSynchronize(s->stream), "create");
        return s;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        destroy(s);
        return nullptr;
    }
}

int monki_cuda_run(void* handle, const uint32_t controls[8], double* out, char* err, size_t errlen) {
    Session* s = static_cast<Session*>(handle);
    if (!s || !controls || !out) { write_error(err, errlen, "Invalid CUDA session or buffers"); return 1; }
    try {
        const Controls c = group_controls(*s, controls);
        execute(*s, c);
        check(cudaMemcpyAsync(out, s->out, size_t(s->layout.count) * c.rounds * sizeof(double), cudaMemcpyDeviceToHost,
                              s->stream), "copy(tallies)");
        finish(*s, c);
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_run_accumulate(void* handle, const uint32_t controls[8], double photons_per_column, double* history,
                              char* err, size_t errlen) {
    Session* s = static_cast<Session*>(handle);
    if (!s || !controls || !history) { write_error(err, errlen, "Invalid CUDA session or buffers"); return 1; }
    try {
        if (!(photons_per_column > 0.0)) throw std::runtime_error("photons_per_column must be positive");
        const Controls c = group_controls(*s, controls);
        execute(*s, c);
        // A failed group must not touch the accumulators: check before accumulating.
        finish(*s, c);
        accumulate(*s, c.rounds, photons_per_column, history);
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

size_t monki_cuda_statistics_count(void* handle) {
    return handle ? statistics_layout(*static_cast<Session*>(handle)).count : 0;
}

int monki_cuda_statistics(void* handle, double* out, size_t count, uint64_t* rounds, char* err, size_t errlen) {
    Session* s = static_cast<Session*>(handle);
    try {
        if (!s || !out || !rounds) throw std::runtime_error("Invalid CUDA session or buffers");
        const StatsLayout L = statistics_layout(*s);
        if (count != L.count) throw std::runtime_error("statistics buffer has the wrong size");
        check(cudaSetDevice(s->device), "cudaSetDevice");
        if (!s->stats) {
            std::fill(out, out + count, 0.0);
        } else {
            check(cudaMemcpyAsync(out, s->stats, count * sizeof(double), cudaMemcpyDeviceToHost, s->stream), "copy(statistics)");
            check(cudaStreamSynchronize(s->stream), "statistics");
        }
        *rounds = s->stats_rounds;
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_reset_statistics(void* handle) {
    Session* s = static_cast<Session*>(handle);
    if (!s) return 1;
    s->stats_rounds = 0;
    if (s->stats) {
        if (cudaSetDevice(s->device) != cudaSuccess) return 1;
        if (cudaMemsetAsync(s->stats, 0, statistics_layout(*s).count * sizeof(double), s->stream) != cudaSuccess) return 1;
    }
    return 0;
}

double monki_cuda_gpu_seconds(void* handle) {
    return handle ? static_cast<Session*>(handle)->gpu_seconds : 0.0;
}

int monki_cuda_last_timing(void* handle, float out[2]) {
    if (!handle || !out) return 1;
    Session* s = static_cast<Session*>(handle);
    out[0] = s->last_kernel_ms;
    out[1] = s->last_run_ms;
    return 0;
}

int monki_cuda_counters(void* handle, uint64_t out[6]) {
    if (!handle || !out) return 1;
    Session* s = static_cast<Session*>(handle);
    for (int q = 0; q < 6; ++q) out[q] = s->totals[q];
    return 0;
}

int monki_cuda_stage_timing(void* handle, double ms[3], uint64_t launches[3]) {
    if (!handle || !ms || !launches) return 1;
    Session* s = static_cast<Session*>(handle);
    for (int q = 0; q < 3; ++q) { ms[q] = s->stage_ms[q]; launches[q] = s->stage_launches[q]; }
    return 0;
}

size_t monki_cuda_tally_count(void* handle) {
    return handle ? static_cast<Session*>(handle)->layout.count : 0;
}

const char* monki_cuda_device_name(void* handle) {
    return handle ? static_cast<Session*>(handle)->name.c_str() : "";
}

void monki_cuda_close(void* handle) { destroy(static_cast<Session*>(handle)); }

int monki_cuda_set_roulette_scale(void* handle, const double* scale, size_t cells, char* err, size_t errlen) {
    Session* s = static_cast<Session*>(handle);
    try {
        if (!s) throw std::runtime_error("Invalid CUDA session");
        const Prepared& p = s->prep;
        const size_t n = size_t(p.nx) * p.ny * p.nz;
        check(cudaSetDevice(s->device), "cudaSetDevice");
        check(cudaStreamSynchronize(s->stream), "sync");
        if (!scale) {
            cudaFree(s->scale);
            s->scale = nullptr;
            return 0;
        }
        if (cells != n) throw std::runtime_error("roulette scale needs nx * ny * nz values");
        for (size_t c = 0; c < n; ++c)
            if (!std::isfinite(scale[c]) || scale[c] < 0.0) throw std::runtime_error("Invalid roulette scale map");
        const size_t elem = s->cfg.fp64 ? sizeof(double) : sizeof(float);
        if (!s->scale) check(cudaMalloc(&s->scale, n * elem), "cudaMalloc(scale)");
        if (s->cfg.fp64) {
            check(cudaMemcpyAsync(s->scale, scale, n * elem, cudaMemcpyHostToDevice, s->stream), "upload(scale)");
            check(cudaStreamSynchronize(s->stream), "upload(scale)");
        } else {
            std::vector<float> f(scale, scale + n);
            check(cudaMemcpyAsync(s->scale, f.data(), n * elem, cudaMemcpyHostToDevice, s->stream), "upload(scale)");
            check(cudaStreamSynchronize(s->stream), "upload(scale)");
        }
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_set_importance_weights(void* handle, const double* weights, size_t pixels, char* err, size_t errlen) {
    Session* s = static_cast<Session*>(handle);
    try {
        if (!s || !s->importance) throw std::runtime_error("The session was created without importance=1");
        const Prepared& p = s->prep;
        const size_t n = size_t(p.nx) * p.ny * p.angles;
        check(cudaSetDevice(s->device), "cudaSetDevice");
        check(cudaStreamSynchronize(s->stream), "sync");
        if (!weights) {
            cudaFree(s->pixel_weight);
            s->pixel_weight = nullptr;
            return 0;
        }
        if (pixels != n) throw std::runtime_error("importance weights need nx * ny * angles values");
        for (size_t c = 0; c < n; ++c)
            if (!std::isfinite(weights[c]) || weights[c] < 0.0) throw std::runtime_error("Invalid importance weights");
        const size_t elem = s->cfg.fp64 ? sizeof(double) : sizeof(float);
        if (!s->pixel_weight) check(cudaMalloc(&s->pixel_weight, n * elem), "cudaMalloc(weights)");
        if (s->cfg.fp64) {
            check(cudaMemcpyAsync(s->pixel_weight, weights, n * elem, cudaMemcpyHostToDevice, s->stream),
                  "upload(weights)");
            check(cudaStreamSynchronize(s->stream), "upload(weights)");
        } else {
            std::vector<float> f(weights, weights + n);
            check(cudaMemcpyAsync(s->pixel_weight, f.data(), n * elem, cudaMemcpyHostToDevice, s->stream),
                  "upload(weights)");
            check(cudaStreamSynchronize(s->stream), "upload(weights)");
        }
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_importance(void* handle, double* out, size_t count, int reset, char* err, size_t errlen) {
    Session* s = static_cast<Session*>(handle);
    try {
        if (!s || !s->importance) throw std::runtime_error("The session was created without importance=1");
        const Prepared& p = s->prep;
        const size_t n = 2 * size_t(p.nx) * p.ny * p.nz;
        if (!out || count != n) throw std::runtime_error("importance needs 2 * nx * ny * nz values");
        check(cudaSetDevice(s->device), "cudaSetDevice");
        check(cudaStreamSynchronize(s->stream), "sync");
        check(cudaMemcpyAsync(out, s->importance, n * sizeof(double), cudaMemcpyDeviceToHost, s->stream),
              "copy(importance)");
        if (reset) check(cudaMemsetAsync(s->importance, 0, n * sizeof(double), s->stream), "memset(importance)");
        check(cudaStreamSynchronize(s->stream), "copy(importance)");
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_inspect(const double* tables, size_t table_count, int fp64, int32_t* uniform_top,
                       double* tau_above, size_t tau_capacity, char* err, size_t errlen) {
    try {
        Prepared p = parse(tables, table_count);
        if (tau_capacity < size_t(p.nz)) throw std::runtime_error("tau_above needs nz values");
        if (fp64) {
            Packed<double> k = pack<double>(p, true);
            *uniform_top = k.uniform_top;
            for (int z = 0; z < p.nz; ++z) tau_above[z] = k.values[k.tau_above + z];
        } else {
            Packed<float> k = pack<float>(p, true);
            *uniform_top = k.uniform_top;
            for (int z = 0; z < p.nz; ++z) tau_above[z] = double(k.values[k.tau_above + z]);
        }
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_inspect_rectangles(const double* tables, size_t table_count, int fp64, uint32_t* extent,
                                  size_t capacity, size_t* written, char* err, size_t errlen) {
    try {
        Prepared p = parse(tables, table_count);
        auto copy = [&](const auto& k) {
            const size_t n = k.extent == SIZE_MAX ? 0 : k.band_count;
            if (n > capacity) throw std::runtime_error("extent needs one word per band cell");
            for (size_t c = 0; c < n; ++c) extent[c] = uint32_t(k.guides[k.extent + c]);
            *written = n;
        };
        if (fp64) copy(pack<double>(p, true));
        else copy(pack<float>(p, true));
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

}  // extern "C"

// ---------------------------------------------------------------------------------------
// Transport without device allocation.
//
// Some callers cannot call cudaMalloc: a host application that hands all device memory
// out of its own arena and forbids other allocations, a real-time pipeline that must not
// allocate (an allocation can synchronize the device or fail under memory pressure) once
// it is running, or a plugin host that owns the GPU's memory budget. For them,
// monki_cuda_run_static runs one round group of the photon-history kernel with every
// scratch buffer (packed scene, FP32 tally bank, failure word, counters, FP64 output
// staging) inside the fixed array below, so the call itself allocates nothing.
//
// The array is 16 MiB, and every GPU that loads this library holds it until the process
// exits. All calls share it and it keeps the last call's contents: each call clears the
// parts that must start at zero, and two calls that overlap on the GPU (from several host
// threads or on several streams) race on it. The first call on a device looks up the
// array's device address for that device and keeps it for the life of the process, so
// make that first call before any stream capture, and do not reset the device
// (cudaDeviceReset) between calls: the kept address would no longer be valid.
// ---------------------------------------------------------------------------------------
namespace monki {
namespace {

constexpr size_t kStaticScratchBytes = size_t(16) << 20;
static __device__ __align__(256) unsigned char g_static_scratch[kStaticScratchBytes];

constexpr int kStaticMaxDevices = 64;
std::mutex g_static_lock;
void* g_static_address[kStaticMaxDevices] = {};
int g_static_grid[kStaticMaxDevices] = {};

}  // namespace
}  // namespace monki

extern "C" int monki_cuda_run_static(uint32_t device, const double* tables, size_t table_count,
                                     const uint32_t controls[8], double* out, char* err, size_t errlen) {
    try {
        if (!tables || !controls || !out) throw std::runtime_error("Invalid tables, controls or output buffer");
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || device >= uint32_t(count) || device >= uint32_t(kStaticMaxDevices))
            throw std::runtime_error("Requested CUDA device is unavailable");
        check(cudaSetDevice(int(device)), "cudaSetDevice");
        void* base = nullptr;
        int grid = 0;
        {
            // Once per device, with the device current: the array's address on this device.
            std::lock_guard<std::mutex> guard(g_static_lock);
            if (!g_static_address[device]) {
                void* address = nullptr;
                check(cudaGetSymbolAddress(&address, g_static_scratch), "cudaGetSymbolAddress");
                cudaDeviceProp prop{};
                check(cudaGetDeviceProperties(&prop, int(device)), "cudaGetDeviceProperties");
                if (prop.major < 10) throw std::runtime_error("This build targets sm_103a (GB300)");
                int blocks = 0;
                check(cudaOccupancyMaxActiveBlocksPerMultiprocessor(
                          &blocks, reinterpret_cast<const void*>(&transport_kernel<float, float, 3, true>), 256, 0),
                      "occupancy");
                g_static_grid[device] = prop.multiProcessorCount * std::max(blocks, 1);
                g_static_address[device] = address;
            }
            base = g_static_address[device];
            grid = g_static_grid[device];
        }

        const Prepared p = parse(tables, table_count);
        if (p.backward || p.nmat == 4)
            throw std::runtime_error("backward transport and nmat 4 need the session API (engine=wavefront)");
        const Controls c{controls[0], controls[1], controls[2], controls[3], controls[4], controls[5], controls[6], controls[7]};
        if (!c.per_round || !c.rounds || !c.max_steps || uint64_t(c.first) + c.count > uint64_t(c.per_round) * c.rounds)
            throw std::runtime_error("Invalid CUDA round group");

        // Layout inside the array: packed scene, tally bank (one shard per round), FP64
        // output staging, mu0/mu per view, failure word and counters.
        Packed<float> k = pack<float>(p, true);
        TallyLayout L{};
        L.stokes = uint32_t(p.nmat * p.nx * p.ny * p.angles);
        L.paths = p.paths ? uint32_t(p.nx * p.ny * p.nz * p.angles) : 0u;
        L.weights = p.paths ? uint32_t(p.nx * p.ny * p.angles) : 0u;
        L.count = L.stokes + L.paths + L.weights;
        L.shards = 1;
        const size_t scene_bytes = align_up(k.values.size() * sizeof(float) + k.guides.size() * sizeof(int), 256);
        const size_t bank_bytes = align_up(size_t(c.rounds) * L.count * sizeof(float), 256);
        const size_t out_bytes = align_up(size_t(c.rounds) * L.count * sizeof(double), 256);
        const size_t mu_bytes = align_up(size_t(p.angles) * sizeof(double), 256);
        const size_t small_bytes = 256;  // failure word + 4 counters
        const size_t needed = scene_bytes + bank_bytes + out_bytes + mu_bytes + small_bytes;
        if (needed > kStaticScratchBytes) {
            char msg[256];
            std::snprintf(msg, sizeof msg,
                          "Scene and round group need %zu bytes of scratch; the static scratch holds %zu (16 MiB)",
                          needed, kStaticScratchBytes);
            throw std::runtime_error(msg);
        }
        char* at = static_cast<char*>(base);
        char* scene = at;
        float* banks = reinterpret_cast<float*>(at + scene_bytes);
        double* staged = reinterpret_cast<double*>(at + scene_bytes + bank_bytes);
        double* mu0mu = reinterpret_cast<double*>(at + scene_bytes + bank_bytes + out_bytes);
        uint32_t* failure = reinterpret_cast<uint32_t*>(at + scene_bytes + bank_bytes + out_bytes + mu_bytes);
        unsigned long long* counters = reinterpret_cast<unsigned long long*>(
            at + scene_bytes + bank_bytes + out_bytes + mu_bytes + 64);

        std::vector<double> mu(size_t(p.angles));
        for (int ia = 0; ia < p.angles; ++ia)
            mu[size_t(ia)] = std::fabs(std::cos(kDegToRad * p.vartheta0)) / std::fabs(std::cos(kDegToRad * p.vartheta[size_t(ia)]));
        check(cudaMemcpy(scene, k.values.data(), k.values.size() * sizeof(float), cudaMemcpyHostToDevice), "upload(scene)");
        if (!k.guides.empty())
            check(cudaMemcpy(scene + k.values.size() * sizeof(float), k.guides.data(), k.guides.size() * sizeof(int),
                             cudaMemcpyHostToDevice), "upload(guides)");
        check(cudaMemcpy(mu0mu, mu.data(), mu.size() * sizeof(double), cudaMemcpyHostToDevice), "upload(mu0mu)");
        // The array keeps the previous call's contents: clear everything that accumulates.
        check(cudaMemset(banks, 0, bank_bytes), "clear(banks)");
        check(cudaMemset(failure, 0, small_bytes), "clear(flags)");
        const SceneView<float> v = make_view<float>(p, k, scene);
        const int blocks = int(std::min<uint64_t>((uint64_t(c.count) + 255) / 256, uint64_t(grid)));
        if (c.count) {
            if (p.nmat == 1 && !p.paths) transport_kernel<float, float, 1, false><<<std::max(blocks, 1), 256>>>(v, c, banks, L, failure, counters);
            else if (p.nmat == 1) transport_kernel<float, float, 1, true><<<std::max(blocks, 1), 256>>>(v, c, banks, L, failure, counters);
            else if (!p.paths) transport_kernel<float, float, 3, false><<<std::max(blocks, 1), 256>>>(v, c, banks, L, failure, counters);
            else transport_kernel<float, float, 3, true><<<std::max(blocks, 1), 256>>>(v, c, banks, L, failure, counters);
            check(cudaGetLastError(), "transport launch");
        }
        const uint64_t total = uint64_t(L.count) * c.rounds;
        const int fgrid = int(std::min<uint64_t>((total + 255) / 256, 4096));
        flush_kernel<float><<<std::max(fgrid, 1), 256>>>(banks, L, p.nmat, p.nx, p.ny, p.nz, p.angles, mu0mu, c.rounds, staged);
        check(cudaGetLastError(), "flush launch");
        uint32_t flag = 0;
        check(cudaMemcpy(&flag, failure, sizeof(flag), cudaMemcpyDeviceToHost), "copy(failure)");
        // A rejected group leaves the caller's buffer untouched.
        if (flag) {
            char msg[128];
            std::snprintf(msg, sizeof msg, "CUDA transport failed (flag %u); round rejected", flag);
            throw std::runtime_error(msg);
        }
        check(cudaMemcpy(out, staged, total * sizeof(double), cudaMemcpyDeviceToHost), "copy(tallies)");
        return 0;
    } catch (const std::exception& e) {
        monki::write_error(err, errlen, e.what());
        return 1;
    }
}
