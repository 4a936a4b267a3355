// Device-resident scene for MONKI photon transport on sm_103a.
//
// The host packer (session.cu) turns the prepared float64 table stream (transport.bin
// v1 of kernels/cpu/worker.f90:1102-1120, or v2 with one azimuth per view) into one
// contiguous device allocation. The kernel receives a SceneView<T> by value; every
// pointer in it points into that allocation.
//
// HBM/L2 layout (T = float for the product build, double for the FP64 check build):
//   cells[4 * cell]          {beta, cumulative fraction of species 1..3} per cell,
//                            cell = i + nx * (j + ny * k), 0-based, k = nz - 1 vacuum
//   zunit[nz], zsum[nz + 1]  layer thickness and its running sum from the surface
//   ssalb_gas[nz], albedo[nx * ny]
//   tau_above[nz]            optical depth of the horizontally uniform layers above k
//   layer_beta[nz]           extinction of a horizontally uniform layer, -1 where it varies
//   vprefix[nz + 1]          vertical optical depth of the uniform layers below each level
//   run_lo[nz], run_hi[nz]   first / last layer of the uniform run containing k (ints)
//   lut_f[4 * n]             {F11, F22, F33, F12} per scattering angle, per species
//   lut_cos[n], lut_cdf[n]   ascending cosine grid and the bound-function CDF
//   lut_v[2 * n]             {F34, F44} per scattering angle, per species (nmat 4 only)
//   guide[kGuide + 1]        CDF guide table: largest i with cdf[i] <= g / kGuide
//   band[nx * ny * uniform_top]  extinction of every cell below the horizontally uniform
//                            top (the only cells a cell walk visits), 16-byte aligned and
//                            padded, staged whole into shared memory when it fits
//   extent[nx * ny * uniform_top]  per band cell, the rectangle of equal-extinction cells
//                            of its layer that holds it (uint32: bytes 0-3 = cells of the
//                            rectangle before it in -x, after it in +x, before it in -y,
//                            after it in +y, each at most 255), from a greedy partition of
//                            every band layer; a straight path inside one rectangle sees a
//                            single extinction, so the free-path walk crosses it in one step
#pragma once
#include <stdint.h>

namespace monki {

constexpr int kMaxViews = 16;
constexpr int kMaxSpecies = 3;
constexpr int kMaxLayers = 64;   // including the vacuum layer
constexpr int kGuide = 4096;
constexpr uint32_t kBandMaxBytes = 48u * 1024u;  // largest band staged in shared memory

// Failure flags shared with the Python host (kernels/metal/README.md:57-59).
enum Failure : uint32_t {
    kNonfinite = 1u,
    kDetectorCap = 2u,
    kSamplingCap = 4u,
    kInvalidStokes = 8u,
    kHistoryCap = 16u,
    kQueueCorrupt = 32u,  // a queue entry outside the photon pool (internal error)
    kStageTimeout = 64u,  // the shared-memory staging copy did not complete in time
};

template <typename T>
struct SceneView {
    int nx, ny, nz, nmat, angles, ntypes, paths, uniform_top;
    int backward;       // backward transport: weight matrices, registration at the injection column
    int lut_n[kMaxSpecies];
    T xunit, yunit, depol;
    T xinv, yinv;        // 1 / xunit, 1 / yunit
    T a0, b0, c0, phi0;  // solar propagation direction cosines and azimuth (rad)
    T inv_mu0;           // 1 / |c0|
    T va[kMaxViews], vb[kMaxViews], vc[kMaxViews], vphi[kMaxViews];
    T vsin[kMaxViews];          // sqrt(max(eps, 1 - vc^2))
    T vcos_phi[kMaxViews], vsin_phi[kMaxViews];  // cos / sin of the view azimuth
    T ssalb_aer[kMaxSpecies];
    T znorm[kMaxSpecies];       // mass of the analog particle sampler (guided weights)
    const T* cells;
    const T* zunit;
    const T* zsum;
    const T* ssalb_gas;
    const T* albedo;
    const T* tau_above;
    const T* layer_beta;
    const T* vprefix;
    const int* run_lo;
    const int* run_hi;
    const T* lut_f[kMaxSpecies];
    const T* lut_cos[kMaxSpecies];
    const T* lut_cdf[kMaxSpecies];
    const int* guide[kMaxSpecies];
    const T* lut_v[kMaxSpecies];  // {F34, F44} per node (nmat 4), else null
    const T* band;          // extinction below the uniform top, i + nx * (j + ny * k)
    uint32_t band_bytes;    // padded size when staged in shared memory, else 0
    const uint32_t* extent; // equal-extinction rectangles of the band cells, or null
};

// Guided transport (detector-directed sampling at particle scatters and Russian
// roulette; see wavefront.cuh). epsilon = 0 and roulette = 0 is the analog method.
template <typename T>
struct Guide {
    T epsilon;         // probability of the detector branch at a particle scatter
    T roulette;        // roulette weight (0 = off), times scale[cell] when a map is set
    T cap;             // detector branch only while the weight is below cap
    const T* scale;    // per-cell roulette scale (nx * ny * nz), or null
    T split;           // split above split x the cell's roulette weight (0 = off)
};

// Splitting: at most kSplitMax copies per split, at most kSplitStack waiting per slot.
constexpr int kSplitMax = 8;
constexpr int kSplitStack = 8;

// Stream of a copy made by splitting: a 32-bit mix of its parent's lineage, the parent's
// draws so far and the copy's index (never 0, the lineage of the photon itself).
__host__ __device__ inline uint32_t split_lineage(uint32_t lineage, uint32_t draws, uint32_t copy) {
    uint32_t h = lineage * 0x9E3779B1u ^ draws * 0x85EBCA77u ^ copy * 0xC2B2AE3Du;
    h ^= h >> 16; h *= 0x85EBCA6Bu; h ^= h >> 13; h *= 0xC2B2AE35u; h ^= h >> 16;
    return h ? h : 1u;
}

// Importance tally of a pilot run: per cell the summed Stokes-I contribution, per unit
// weight at the event, of the event and the next kRing - 1 events of its history, then
// the event count (2 * nx * ny * nz FP64 values).
constexpr int kRing = 8;

// Per-launch controls, the eight words of the Metal ABI v2 (kernels/metal/README.md:52-55).
struct Controls {
    uint32_t count, first, first_round, seed, max_steps, profile, per_round, rounds;
};

// The largest history step limit (max_steps) a session accepts; a count up to it is exact
// in FP32, where walks without layer paths keep it.
constexpr uint32_t kMaxHistorySteps = 10000000u;

// Device tally layout of one round and one shard (TA = float or double):
//   stokes[m + nmat * (i + nx * (j + ny * ia))]
//   paths [k + nz * (i + nx * (j + ny * ia))]      k contiguous for vector reductions
//   weights[i + nx * (j + ny * ia)]
struct TallyLayout {
    uint32_t stokes, paths, weights, count;  // element counts; count = sum
    uint32_t shards;
    uint32_t orders;  // scattering-order diagnostics after the weights (0 = off):
                      // single-scattering Stokes (stokes elements), then the contribution of
                      // every event location and its single-scattering part
                      // (nmat * nx * ny * nz * angles each, layer 0 = the surface)
};

}  // namespace monki
