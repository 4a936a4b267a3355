// Wavefront transport for MONKI on sm_103a: photon state lives in a device pool and each
// stage of a history runs as its own kernel over event queues, so a warp always executes
// one kind of work.
//
//   transit  walks every pooled photon along its free path (ADVANCE, mc.f90:1531-1580)
//            to its next interaction, draws the species and applies the single-scattering
//            albedo (mc.f90:1028-1074) or the surface albedo (mc.f90:681-728), and appends
//            the photon to the surface / gas / particle queue. Slots whose photon escaped or
//            died claim the next photon of the round group, so the pool stays full.
//            Horizontally uniform layer runs are crossed in one jump with a vertical
//            optical-depth prefix; a per-launch step budget keeps the lanes of a warp in step.
//   peel     one thread per event, all views: phase matrix and rotations, optical depth to
//            the top along each view (calc_radiances_and_paths_pol,
//            mc_routines_cartesian_mod.f90:849-1222) and the tallies, as 128-bit atomics.
//   scatter  Lambertian reflection (GROUND_LAMB2) or polarized rejection sampling of the
//            new direction with the Stokes update (mc.f90:1266-1431), then roulette and
//            splitting of guided transport.
//   step     (scenes without layer paths; the default there) scatter and transit fused:
//            from double-buffered work lists (the three event queues, the walks paused by
//            the step budget, the vacant slots), each queued event is scattered and its
//            photon walks on to its next event in the same thread, filing the slot in the
//            other buffer's lists. One iteration is then step + peel.
//   tail     the end of a round group: once every photon is claimed and few remain, one
//            resident wave runs each remaining photon to its end with the same per-slot
//            walk, peel-off and scattering functions.
//
// Photon state is stored as 16-byte records per slot (position, direction, polarization,
// bookkeeping), one load or store per record.
//
// Each photon's random stream is addressed by a draw index, so the draw sequence of a
// history is the same as in one thread (and as in the CPU oracle) however the stages split.
//
// Layer-path (AMF) tallies are decomposed exactly: a history's path per layer is the
// straight initial descent (whole layers above the first event at 1/|mu0|, a partial piece
// in the first-event layer), then the wandering after it, and each detector ray adds whole
// layers above the event at 1/mu plus a partial piece. The straight parts are tallied as
// one weight per (pixel, first layer) and are expanded by a prefix sum in the FP64 flush;
// only the wandering range is tallied layer by layer.
#pragma once
#include "transport.cuh"

namespace monki {

constexpr uint32_t kNone = 0xFFFFFFFFu;

enum Queue : int { kQueueSurface = 0, kQueueGas = 1, kQueueParticle = 2 };

template <typename T>
struct alignas(4 * sizeof(T)) Quad { T x, y, z, w; };

// Unsigned division by a launch constant with one multiply-high and two shifts
// (round-up method; d == 1 handled separately).
struct FastDiv {
    uint32_t d, m, l;
    __host__ static FastDiv make(uint32_t d) {
        FastDiv f{d, 0u, 0u};
        if (d > 1) {
            uint32_t l = 0;
            while ((uint64_t(1) << l) < d) ++l;
            f.l = l;
            f.m = uint32_t((((uint64_t(1) << 32) * ((uint64_t(1) << l) - d)) / d) + 1);
        }
        return f;
    }
    __device__ __forceinline__ uint32_t div(uint32_t n) const {
        if (d == 1) return n;
        const uint32_t t = __umulhi(m, n);
        return (t + ((n - t) >> 1)) >> (l - 1);
    }
    __device__ __forceinline__ uint32_t mod(uint32_t n) const { return n - div(n) * d; }
};

struct Divisors { FastDiv per_round, nx, ny, ncol; };

// Device tally layout of one round and one shard (element counts of TA):
//   pixel records  [pixel]                  {I, Q, U, detected weight}
//   layer records  [pixel * 2 * span + k]   path pieces tallied per layer: the wander, the
//                                           partial view ray and the partial initial descent
//                  [pixel * 2 * span + span + k]
//                                           difference array of the straight paths per unit
//                                           layer thickness: +w / mu_view above the event layer,
//                                           +w / |mu0| above the first-event layer (from layer 0
//                                           when the surface came first), and each straight run
//                                           of whole layers, +w / |cos| from its first layer and
//                                           -w / |cos| past its last
//   span = nz + 1 rounded up to a multiple of 4, so one 128-bit atomic covers four layers
//   (L2 atomics cost per request, not per byte); element nz of the path array holds
//   w / mu_view of events in the top layer, whose view rays cross no whole layer.
struct WaveTally {
    uint32_t pixels;   // nx * ny * angles
    uint32_t span;     // per-pixel length of each layer array: nz + 1 rounded up to a multiple of 4
    uint32_t layers;   // pixels * 2 * span when paths are tallied, else 0
    uint32_t count;    // 4 * pixels + layers (+ the order records)
    uint32_t shards;
    // Scattering-order diagnostics (0 = off): element offset of the single-scattering
    // pixel records {I, Q, U, -} (pixels), followed by the location records {I, Q, U, -} of
    // every (column, layer, view), cell = i + nx (j + ny (layer + nz view)), layer 0 = the
    // surface, then their single-scattering part.
    uint32_t orders;
    uint32_t locations;  // nx * ny * nz * angles
    // Circular polarization (nmat 4): element offset of one V record per pixel (the pixel
    // records hold {I, Q, U, path weight}); order records carry V in their fourth element.
    uint32_t vee;
};

// A photon copy made by splitting, waiting in its slot: the records of the pool, one
// 64-byte block in FP32 — {photon id, the copy's stream lineage (its draws start at 0),
// cell | kind, packed layers}, position, direction, and {Q, U, V in place of the free path
// (which the copy draws anew), the step count} (splitting runs only in scenes without layer
// paths, whose slots keep the step count there too). With order tallies the history's
// scattering order goes beside it in Pool::copy_order.
template <typename T>
struct SplitCopy {
    uint4 meta;
    Quad<T> pos, dir, pol;
};

// Resident blocks of 256 per SM the fused step kernel is built for (its register budget,
// 65536 / (256 x blocks)); a build option for measuring the trade of occupancy for spills.
#ifndef MONKI_STEP_BLOCKS
#define MONKI_STEP_BLOCKS 4
#endif

constexpr uint32_t kListCounts = 8;   // counts per work-list buffer
constexpr uint32_t kClaimCount = 16;  // index of the claim counter
constexpr uint32_t kCountWords = 20;  // words of the counts array

// Bytes of one slot's state block: three records of four T and the bookkeeping record.
template <typename T>
constexpr size_t kRecordBytes = sizeof(T) == 4 ? 64 : 128;

// Bookkeeping word of a slot's cell and pending event: i | j << 12 | kind << 24, with kind
// 0 gas, 1 + s particle species s, 255 surface (grids up to 4096 columns a side).
__host__ __device__ __forceinline__ uint32_t pack_cell(int i, int j, int kind) {
    return uint32_t(i) | (uint32_t(j) << 12) | (uint32_t(kind) << 24);
}
__host__ __device__ __forceinline__ int cell_i(uint32_t w) { return int(w & 0xFFFu); }
__host__ __device__ __forceinline__ int cell_j(uint32_t w) { return int((w >> 12) & 0xFFFu); }
__host__ __device__ __forceinline__ int cell_kind(uint32_t w) { return int(w >> 24); }
constexpr int kMaxColumnsPerAxis = 4096;

template <typename T>
struct Pool {
    uint32_t capacity;
    // Per slot one block of kRecordBytes<T>: position {x, y, z, weight}, direction {a, b, c,
    // phi}, polarization {q, u, remains, init_part}, bookkeeping {pid (kNone when empty),
    // next draw, pack_cell(i, j, pending event kind), packed layers}. The four records of a
    // slot are read and written together, so its accesses fill whole 32-byte sectors.
    unsigned char* records;
    // Walk steps so far (the history step limit), one word per slot in scenes with layer
    // paths; null in scenes without them, where the count rides in the polarization record's
    // fourth element (init_part, unused there) as an exact FP value (at most 10^7 + 1 steps),
    // so a walk reads and writes its slot's 64-byte block and nothing else.
    uint32_t* steps;
    T* wander;       // capacity * nz path lengths after the first event
    uint32_t* runs;  // two straight runs of whole layers: lo0 | hi0 << 8 | lo1 << 16 | hi1 << 24
    T* run_ci;       // capacity * 2: 1 / |cos| of each run
    // Work lists of a wavefront iteration, double buffered (b = 0, 1): the event queues
    // (surface, gas, particle), the photons paused mid-walk and the empty slots to fill.
    // A step launch reads buffer b and writes buffer 1 - b; the peel-off reads the events
    // the step wrote.
    uint32_t* queue[2][3];
    uint32_t* paused[2];
    uint32_t* vacant[2];
    // counts[kListCounts * b + ...]: [0..2] queue sizes, [3] paused, [4] vacant slots of
    // buffer b; counts[kClaimCount]: the next photon to claim. A photon is live exactly
    // when its slot is queued or paused, or holds waiting split copies.
    uint32_t* counts;
    // Importance tally (pilot runs only; null otherwise): the cells and 1 / weight of the
    // last kRing events of each history, and the per-cell FP64 sums.
    uint32_t* ring_cell;  // capacity * kRing
    T* ring_inv;          // capacity * kRing
    uint32_t* ring_n;     // events so far
    double* importance;   // 2 * nx * ny * nz
    const T* pixel_weight;  // nx * ny * angles weights of the contributions, or null (all 1)
    uint32_t* order;      // events so far of each slot's history (scattering-order tallies), or null
    T* vee;               // V of the normalized Stokes vector (forward nmat 4), or null
    // Backward transport: the weight matrix of each history, nmat * nmat elements
    // (row-major, M11 = 1 after normalization), element e of slot s at matrix[e * capacity + s].
    T* matrix;
    uint32_t* first;      // backward with order tallies: the first event's cell (i | j << 12 | layer << 24)
    // Splitting (null when off): each slot's stream lineage, its waiting copies (copy c of
    // slot s at copies[s * kSplitStack + c]) and their count.
    uint32_t* lineage;
    SplitCopy<T>* copies;
    uint32_t* copy_order;  // scattering order of each waiting copy with order tallies, else null
    uint32_t* waiting;

    __device__ __forceinline__ Quad<T>& pos(uint32_t s) const {
        return *reinterpret_cast<Quad<T>*>(records + size_t(s) * kRecordBytes<T>);
    }
    __device__ __forceinline__ Quad<T>& dir(uint32_t s) const {
        return *reinterpret_cast<Quad<T>*>(records + size_t(s) * kRecordBytes<T> + sizeof(Quad<T>));
    }
    __device__ __forceinline__ Quad<T>& pol(uint32_t s) const {
        return *reinterpret_cast<Quad<T>*>(records + size_t(s) * kRecordBytes<T> + 2 * sizeof(Quad<T>));
    }
    __device__ __forceinline__ uint4& meta(uint32_t s) const {
        return *reinterpret_cast<uint4*>(records + size_t(s) * kRecordBytes<T> + 3 * sizeof(Quad<T>));
    }
};

// A slot's four records, handed from the scattering to the walk in registers.
template <typename T>
struct SlotState {
    uint4 meta;
    Quad<T> pos, dir, pol;
};

__device__ __forceinline__ uint32_t pack_layers(int k, int k1, int wmin, int wmax) {
    return uint32_t(k + 1) | (uint32_t(k1 + 2) << 8) | (uint32_t(wmin) << 16) | (uint32_t(wmax) << 24);
}
__device__ __forceinline__ void unpack_layers(uint32_t v, int& k, int& k1, int& wmin, int& wmax) {
    k = int(v & 0xFF) - 1;
    k1 = int((v >> 8) & 0xFF) - 2;
    wmin = int((v >> 16) & 0xFF);
    wmax = int(v >> 24);
}

// Stage the extinction band (every cell below the uniform top) into this block's shared
// memory with one bulk asynchronous copy (TMA engine) completing on an mbarrier. Returns
// the shared copy, or null when the band is not staged (too large, or absent) or the copy
// did not complete within the wait limit (then kStageTimeout is raised and the caller
// reads global memory). Every thread of the block must call it.
template <typename T>
__device__ __forceinline__ const T* stage_band(const SceneView<T>& s, unsigned char* smem, uint32_t* failure) {
    if (!s.band_bytes) return nullptr;
    __shared__ __align__(8) uint64_t barrier;
    const uint32_t bar = uint32_t(__cvta_generic_to_shared(&barrier));
    const uint32_t dst = uint32_t(__cvta_generic_to_shared(smem));
    if (threadIdx.x == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar), "r"(s.band_bytes) : "memory");
        asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
                     ::"r"(dst), "l"(s.band), "r"(s.band_bytes), "r"(bar) : "memory");
    }
    __syncthreads();
    uint32_t done = 0;
    for (uint32_t attempt = 0; attempt < (1u << 22) && !done; ++attempt) {
        asm volatile(
            "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.b32 %0, 1, 0, p;\n}"
            : "=r"(done) : "r"(bar) : "memory");
    }
    if (!done) {
        if (threadIdx.x == 0) atomicOr(failure, kStageTimeout);
        // The copy may still be in flight: give it a second bounded wait before the block goes
        // on without the staged band (a later landing only touches the unused staging area).
        for (uint32_t attempt = 0; attempt < (1u << 22) && !done; ++attempt) {
            asm volatile(
                "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.b32 %0, 1, 0, p;\n}"
                : "=r"(done) : "r"(bar) : "memory");
        }
        return nullptr;
    }
    return reinterpret_cast<const T*>(smem);
}

// Extinction of a cell below the uniform top: the staged copy when there is one.
template <typename T>
__device__ __forceinline__ T band_beta(const SceneView<T>& s, const T* band, int i, int j, int k) {
    return band ? band[i + s.nx * (j + s.ny * k)] : beta_at(s, i, j, k);
}

// A photon's Philox stream addressed by draw index: draw d is word d % 4 of block d / 4.
struct DrawStream {
    uint32_t photon, round, seed, draw, loaded, lineage;
    uint4 words;
    // lineage: 0 for the photon itself, a split copy's own value otherwise (the fourth
    // counter word).
    __device__ __forceinline__ void init(uint32_t p, uint32_t r, uint32_t s, uint32_t d, uint32_t l = 0u) {
        photon = p; round = r; seed = s; draw = d; loaded = kNone; lineage = l;
    }
    __device__ __forceinline__ float next() {
        const uint32_t blk = draw >> 2;
        if (blk != loaded) {
            words = philox4x32_10(make_uint4(photon, round, blk, lineage), make_uint2(seed, 0u));
            loaded = blk;
        }
        const uint32_t lane = draw & 3u;
        const uint32_t w = lane == 0 ? words.x : lane == 1 ? words.y : lane == 2 ? words.z : words.w;
        ++draw;
        return (float(w >> 9) + 0.5f) * 0x1p-23f;
    }
};

// Reserve one entry of counters[key] per calling lane. Lanes that arrive together are
// grouped by key, so each counter advances only by the lanes that write to its queue.
__device__ __forceinline__ uint32_t warp_reserve(uint32_t* counters, int key = 0) {
    const uint32_t active = __activemask();
    const uint32_t group = __match_any_sync(active, key);
    const int leader = __ffs(group) - 1;
    const uint32_t lane = threadIdx.x & 31u;
    uint32_t base = 0;
    if (int(lane) == leader) base = atomicAdd(counters + key, uint32_t(__popc(group)));
    base = __shfl_sync(group, base, leader);
    return base + uint32_t(__popc(group & ((1u << lane) - 1u)));
}

// Sum N per-thread counters over the block and add each nonzero total to its target from
// one thread. Per-warp atomics on a few shared addresses serialize in L2: tens of
// thousands of them cost a launch over ten microseconds even when it has no work.
template <int N, typename U>
__device__ __forceinline__ void block_add(const unsigned long long (&v)[N], U* const (&target)[N]) {
    __shared__ unsigned long long part[N][32];
    const int warp = int(threadIdx.x >> 5), lane = int(threadIdx.x & 31);
    const int warps = int((blockDim.x + 31) >> 5);
#pragma unroll
    for (int q = 0; q < N; ++q) {
        unsigned long long x = v[q];
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
        if (lane == 0) part[q][warp] = x;
    }
    __syncthreads();
    if (warp == 0) {
#pragma unroll
        for (int q = 0; q < N; ++q) {
            unsigned long long x = lane < warps ? part[q][lane] : 0ull;
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) x += __shfl_down_sync(0xffffffffu, x, off);
            if (lane == 0 && x) atomicAdd(target[q], U(x));
        }
    }
}

// Add v to the wander entry of layer kk, keeping [wmin, wmax] the only valid range:
// entries newly covered by the range are zeroed first, so a new photon needs no clearing.
template <typename T>
__device__ __forceinline__ void wander_add(T* w, int kk, T v, int& wmin, int& wmax) {
    if (wmin > wmax) {
        w[kk] = v;
        wmin = wmax = kk;
    } else if (kk > wmax) {
        for (int q = wmax + 1; q < kk; ++q) w[q] = T(0);
        w[kk] = v;
        wmax = kk;
    } else if (kk < wmin) {
        for (int q = kk + 1; q < wmin; ++q) w[q] = T(0);
        w[kk] = v;
        wmin = kk;
    } else {
        w[kk] += v;
    }
}

// The layer-path record of a photon after its first event: partial-layer lengths in the
// wander range, and up to two straight runs of whole layers crossed in uniform runs (each
// whole layer m of a run adds zunit[m] / |cos|), tallied later as a difference array.
// A third run falls back to the wander array.
constexpr uint32_t kNoRuns = 0xFFFFFFFFu;

template <typename T>
struct PathRecord {
    T* wander;
    int wmin, wmax;
    uint32_t runs;
    T ci0, ci1;
    __device__ __forceinline__ void add(int kk, T v) { wander_add(wander, kk, v, wmin, wmax); }
    __device__ __forceinline__ void run(const T* zunit, int lo, int hi, T ci) {
        if ((runs & 0xFFu) == 0xFFu) {
            runs = (runs & 0xFFFF0000u) | uint32_t(lo) | (uint32_t(hi) << 8);
            ci0 = ci;
        } else if (((runs >> 16) & 0xFFu) == 0xFFu) {
            runs = (runs & 0x0000FFFFu) | (uint32_t(lo) << 16) | (uint32_t(hi) << 24);
            ci1 = ci;
        } else {
            for (int m = lo; m <= hi; ++m) add(m, __ldg(zunit + m) * ci);
        }
    }
};

// Move a distance h >= 0 along one horizontal axis of the periodic grid: x is the distance
// to the next face in direction sgn, inv = 1 / unit. Equivalent to the face-by-face walk
// of ADVANCE: the whole cells crossed come from one multiply, corrected by one cell either
// way, and a face hit to rounding leaves the photon on the face.
template <typename T>
__device__ __forceinline__ void slide(int& i, T& x, int sgn, T h, T unit, T inv, int n) {
    if (h < x) { x = x - h; return; }
    T rest = h - x;
    T whole = floor(rest * inv);
    rest -= whole * unit;
    // 32-bit counts: no float-to-int64 conversion or 64-bit modulo (slow conversion and
    // FP64-pipe work on this GPU); 4e9 faces exceed any travel a float position resolves.
    uint32_t cross = 1u + uint32_t(fmin(whole, T(4.0e9)));
    if (rest < T(0)) { rest += unit; --cross; if (rest < T(0)) rest = T(0); }
    if (rest >= unit) { rest -= unit; ++cross; }
    const int step = int(cross < uint32_t(n) ? cross : cross % uint32_t(n));
    i += sgn * step;
    i = i < 0 ? i + n : (i >= n ? i - n : i);
    x = unit - rest;
}

// Along one horizontal axis inside an equal-extinction rectangle: a slide when the
// rectangle reaches beyond the current cell (extra > 0), else the in-cell step of advance.
template <typename T>
__device__ __forceinline__ void move_within(int& i, T& x, int sgn, T h, T unit, T inv, int n, int extra) {
    if (extra) slide(i, x, sgn, h, unit, inv, n);
    else x = fmax(T(0), x - h);
}

// Whole cells of the equal-extinction rectangle around band cell (i, j, k) beyond the
// current one in the direction of travel: ex along x, ey along y (0 without rectangles).
template <typename T>
__device__ __forceinline__ void rectangle_reach(const SceneView<T>& s, int i, int j, int k, int is, int js, int& ex,
                                                int& ey) {
    ex = 0; ey = 0;
    if (s.extent) {
        const uint32_t w = __ldg(s.extent + i + s.nx * (j + s.ny * k));
        ex = int((w >> (is > 0 ? 8 : 0)) & 0xFFu);
        ey = int((w >> (js > 0 ? 24 : 16)) & 0xFFu);
    }
}

// advance through an equal-extinction rectangle: to its nearest face in one step. A
// straight path inside the rectangle meets one extinction, so this is the face-by-face
// walk of ADVANCE with the interior faces skipped; with ex = ey = 0 it is advance exactly.
template <typename T>
__device__ __forceinline__ T advance_rectangle(const SceneView<T>& s, int& i, int& j, int& k, T& x, T& y, T& z,
                                               int is, int js, int ks, T aa, T ba, T ca, T ai, T bi, T ci, int ex,
                                               int ey) {
    const T dx = (ex ? x + T(ex) * s.xunit : x) * ai;
    const T dy = (ey ? y + T(ey) * s.yunit : y) * bi;
    const T dz = z * ci;
    const T dist = fmin(dx, fmin(dy, dz));
    if (dx == dist) {
        // The rectangle lies inside the grid, so one wrap brings i back into [0, nx).
        i += is * (ex + 1); i = i < 0 ? i + s.nx : (i >= s.nx ? i - s.nx : i);
        x = s.xunit;
        move_within(j, y, js, ba * dist, s.yunit, s.yinv, s.ny, ey);
        z = fmax(T(0), z - ca * dist);
    } else if (dy == dist) {
        j += js * (ey + 1); j = j < 0 ? j + s.ny : (j >= s.ny ? j - s.ny : j);
        move_within(i, x, is, aa * dist, s.xunit, s.xinv, s.nx, ex);
        y = s.yunit;
        z = fmax(T(0), z - ca * dist);
    } else {
        k += ks;
        move_within(i, x, is, aa * dist, s.xunit, s.xinv, s.nx, ex);
        move_within(j, y, js, ba * dist, s.yunit, s.yinv, s.ny, ey);
        if (k >= 0 && k < s.nz) z = __ldg(s.zunit + k);
    }
    return dist;
}

// One jump through the horizontally uniform run that contains layer k, from the current
// position (z: vertical distance to the exit face in direction ks). Returns 0 for an
// interaction inside the run, 1 for the surface, 2 for escape through the top, and -1
// when the photon enters a horizontally varying layer (at its face, z = zunit). Path
// lengths per layer go to the wander array when `record`; an escaping photon needs none.
template <typename T>
__device__ __forceinline__ int uniform_jump(const SceneView<T>& s, int& k, T& z, T& remains, int ks, T ca, T ci,
                                            bool record, PathRecord<T>& path,
                                            int& i, T& x, int is, T aa, int& j, T& y, int js, T ba) {
    const T eps = Tol<T>::eps;
    const int top = s.nz - 1;
    int outcome;
    T travelled;
    const T bk = __ldg(s.layer_beta + k);
    const T seg = z * ci;
    if (bk > eps && remains / bk < seg) {
        const T de = remains / bk;
        travelled = de;
        z = fmax(T(0), z - ca * de);
        if (record) path.add(k, de);
        outcome = 0;
    } else {
        remains -= seg * bk;
        travelled = seg;
        if (record) path.add(k, seg);
        const int m0 = k + ks;
        // Layers m0 .. end of the run, in the direction of travel.
        const int end = ks > 0 ? __ldg(s.run_hi + k) : __ldg(s.run_lo + k);
        const T* V = s.vprefix;   // V[m] = vertical optical depth of uniform layers below m
        const T* Z = s.zsum;      // Z[m] = height of the bottom of layer m
        const bool inside = ks > 0 ? m0 <= end : m0 >= end;
        const T run_tau = !inside ? T(0) : (ks > 0 ? __ldg(V + end + 1) - __ldg(V + m0) : __ldg(V + m0 + 1) - __ldg(V + end));
        if (!inside || remains * ca >= run_tau) {
            // Leaves the run: every remaining layer of it is crossed whole.
            if (inside) {
                remains -= run_tau * ci;
                const T height = ks > 0 ? __ldg(Z + end + 1) - __ldg(Z + m0) : __ldg(Z + m0 + 1) - __ldg(Z + end);
                travelled += height * ci;
            }
            k = inside ? end + ks : m0;
            if (k > top) outcome = 2;
            else outcome = k < 0 ? 1 : -1;
            if (outcome != 2 && record && inside) path.run(s.zunit, min(m0, end), max(m0, end), ci);
            if (outcome == -1) z = __ldg(s.zunit + k);
        } else {
            // The interaction lies inside the run: find its layer m, the first one (from
            // m0 in the direction of travel) whose vertical optical depth, summed from m0,
            // exceeds need. A binary search over the prefix V: about log2 of the run
            // length steps for every lane, where a layer-by-layer scan diverged across
            // the warp with runs of up to nz layers.
            const T need = remains * ca;
            int m;
            T before;  // vertical optical depth of the whole layers crossed before m
            if (ks > 0) {
                const T v0 = __ldg(V + m0);
                int lo = m0, hi = end;
                while (lo < hi) {
                    const int mid = (lo + hi) >> 1;
                    if (__ldg(V + mid + 1) - v0 > need) hi = mid;
                    else lo = mid + 1;
                }
                m = lo;
                before = __ldg(V + m) - v0;
            } else {
                const T v0 = __ldg(V + m0 + 1);
                int lo = end, hi = m0;
                while (lo < hi) {
                    const int mid = (lo + hi + 1) >> 1;
                    if (v0 - __ldg(V + mid) > need) lo = mid;
                    else hi = mid - 1;
                }
                m = lo;
                before = v0 - __ldg(V + m + 1);
            }
            const T slant_before = (ks > 0 ? __ldg(Z + m) - __ldg(Z + m0) : __ldg(Z + m0 + 1) - __ldg(Z + m + 1)) * ci;
            remains -= before * ci;
            const T bm = __ldg(s.layer_beta + m);
            const T de = bm > eps ? remains / bm : T(0);
            travelled += slant_before + de;
            if (record) {
                if (m != m0) path.run(s.zunit, min(m0, m - ks), max(m0, m - ks), ci);
                path.add(m, de);
            }
            k = m;
            z = fmax(T(0), __ldg(s.zunit + m) - ca * de);
            outcome = 0;
        }
    }
    if (outcome != 2) {
        slide(i, x, is, aa * travelled, s.xunit, s.xinv, s.nx);
        slide(j, y, js, ba * travelled, s.yunit, s.yinv, s.ny);
    }
    return outcome;
}

// ----------------------------------------------------------------------------------
// transit: free path to the next interaction for every pooled photon.
// ----------------------------------------------------------------------------------
// One slot's walk to its next event: continues a split copy or claims a photon into an
// empty slot (when claims are open), walks it, selects the interaction and stores the
// state. Returns the event's queue (surface, gas, particle) or -1 when the slot holds no
// event (empty, finished, or paused by the step budget). QUEUE files the slot in the work
// lists of buffer `out` (its event queue, the paused list, or the vacant list while it can
// still be filled); without it the caller handles the event (the tail kernel). `given`
// holds the slot's records when the caller has them in registers (a scattering just
// made them); they are then not read back from memory.
template <typename T, bool PATHS, bool QUEUE>
__device__ __forceinline__ int transit_slot(uint32_t slot, const SceneView<T>& s, const T* band, const Controls& ctl,
                                            const Divisors& dv, const Pool<T>& P, uint32_t walk, bool may_claim,
                                            uint32_t out, uint32_t* __restrict__ failure, uint64_t& scatters,
                                            uint64_t& visits, const SlotState<T>* given = nullptr) {
    const T eps = Tol<T>::eps;
    const int top = s.nz - 1;
    int event = -1;
    // All records at once, before the empty-slot test: one memory latency instead of two.
    uint4 meta;
    Quad<T> pos_in, dir_in, pol_in;
    if (given) {
        meta = given->meta; pos_in = given->pos; dir_in = given->dir; pol_in = given->pol;
    } else {
        meta = P.meta(slot); pos_in = P.pos(slot); dir_in = P.dir(slot); pol_in = P.pol(slot);
    }
    const uint32_t steps_in = P.steps ? P.steps[slot] : uint32_t(pol_in.w);
    uint32_t pid = meta.x;
    DrawStream rng;
    int i = 0, j = 0, k = 0, k1 = -2, wmin = 255, wmax = 0;
    Quad<T> pos{}, dir{}, pol{};
    uint32_t steps = 0, budget = walk, order = 0;
    bool fresh = false;
    PathRecord<T> path{PATHS ? P.wander + size_t(slot) * s.nz : nullptr, 255, 0, kNoRuns, T(0), T(0)};

    uint32_t lineage = 0u;
    if (pid != kNone) {
        const uint32_t ro = dv.per_round.div(pid);
        if (P.lineage) lineage = P.lineage[slot];
        rng.init(pid - ro * ctl.per_round, ctl.first_round + ro, ctl.seed, meta.y, lineage);
        i = cell_i(meta.z); j = cell_j(meta.z);
        unpack_layers(meta.w, k, k1, wmin, wmax);
        pos = pos_in;
        dir = dir_in;
        pol = pol_in;
        steps = steps_in;
        if (P.order) order = P.order[slot];
        if (PATHS) {
            path.runs = P.runs[slot];
            path.ci0 = P.run_ci[2 * size_t(slot)];
            path.ci1 = P.run_ci[2 * size_t(slot) + 1];
        }
    }
    path.wmin = wmin; path.wmax = wmax;
    T& x = pos.x; T& y = pos.y; T& z = pos.z; T& weight = pos.w;
    T& remains = pol.z; T& init_part = pol.w;

    T vee = T(0);
    int pending = 0;  // the event's kind, kept in the bookkeeping record
    for (;;) {
        if (pid == kNone && P.waiting && P.waiting[slot] > 0u) {
            // A copy left by splitting continues in this slot, with its own stream and a
            // new free path drawn from it.
            const uint32_t n = P.waiting[slot] - 1u;
            const size_t entry = size_t(slot) * kSplitStack + n;
            const SplitCopy<T> cp = P.copies[entry];
            P.waiting[slot] = n;
            pid = cp.meta.x;
            lineage = cp.meta.y;
            i = cell_i(cp.meta.z); j = cell_j(cp.meta.z);
            unpack_layers(cp.meta.w, k, k1, wmin, wmax);
            path.wmin = wmin; path.wmax = wmax;
            pos = cp.pos; dir = cp.dir; pol = cp.pol;
            steps = uint32_t(cp.pol.w);
            order = P.copy_order ? P.copy_order[entry] : 0u;
            vee = cp.pol.z;
            const uint32_t ro = dv.per_round.div(pid);
            rng.init(pid - ro * ctl.per_round, ctl.first_round + ro, ctl.seed, 0u, lineage);
            remains = -log(fmax(T(rng.next()), eps));
            fresh = true;
        }
        if (pid == kNone) {
            // Read first so a drained group stops reserving (the counter never wraps).
            if (!may_claim || *reinterpret_cast<volatile uint32_t*>(P.counts + kClaimCount) >= ctl.count) break;
            const uint32_t n = warp_reserve(P.counts + kClaimCount);
            if (n >= ctl.count) break;
            pid = ctl.first + n;
            const uint32_t ro = dv.per_round.div(pid);
            const uint32_t photon = pid - ro * ctl.per_round;
            rng.init(photon, ctl.first_round + ro, ctl.seed, 0u);
            const uint32_t column = dv.ncol.mod(photon);
            const uint32_t row = dv.nx.div(column);
            i = int(column - row * uint32_t(s.nx));
            j = min(int(row), s.ny - 1);
            k = top;
            x = s.xunit * T(rng.next());
            y = s.yunit * T(rng.next());
            z = __ldg(s.zunit + k);
            weight = T(1);
            order = 0;
            dir = Quad<T>{s.a0, s.b0, s.c0, s.phi0};
            pol.x = T(0); pol.y = T(0);
            steps = 0;
            k1 = -2; init_part = T(0);
            path.wmin = 255; path.wmax = 0; path.runs = kNoRuns;
            remains = -log(fmax(T(rng.next()), eps));
            lineage = 0u; vee = T(0);
            fresh = true;
        }
        const T a = dir.x, b = dir.y, c = dir.z;
        const int is = signbit(a) ? -1 : 1, js = signbit(b) ? -1 : 1, ks = signbit(c) ? -1 : 1;
        const T aa = fabs(a), ba = fabs(b), ca = fabs(c);
        const T ai = T(1) / fmax(aa, eps), bi = T(1) / fmax(ba, eps), ci = T(1) / fmax(ca, eps);
        // Path length of the current layer, added to the wander array on layer change.
        const bool record = PATHS && k1 > -2;
        int acc_k = -1;
        T acc = T(0);
        int outcome = -1;  // 0 atmosphere, 1 surface, 2 escaped, 3 step limit, 4 paused
        for (;;) {
            if (budget == 0) { outcome = 4; break; }
            --budget;
            if (++steps > ctl.max_steps) { outcome = 3; break; }
            ++visits;
            if (__ldg(s.layer_beta + k) >= T(0)) {
                outcome = uniform_jump<T>(s, k, z, remains, ks, ca, ci, record, path, i, x, is, aa, j, y, js, ba);
                if (outcome >= 0) break;
                continue;
            }
            const T bv = k < top ? band_beta<T>(s, band, i, j, k) : T(0);
            int ex = 0, ey = 0;
            if (k < top) rectangle_reach(s, i, j, k, is, js, ex, ey);
            if (bv > eps) {
                const T de = remains / bv;
                if (de < (ex ? x + T(ex) * s.xunit : x) * ai && de < (ey ? y + T(ey) * s.yunit : y) * bi &&
                    de < z * ci) {
                    move_within(i, x, is, aa * de, s.xunit, s.xinv, s.nx, ex);
                    move_within(j, y, js, ba * de, s.yunit, s.yinv, s.ny, ey);
                    z = fmax(T(0), z - ca * de);
                    if (record) {
                        if (acc_k != k) {
                            if (acc_k >= 0) path.add(acc_k, acc);
                            acc_k = k; acc = T(0);
                        }
                        acc += de;
                    }
                    outcome = 0;
                    break;
                }
            }
            const int k_old = k;
            const T dist = advance_rectangle(s, i, j, k, x, y, z, is, js, ks, aa, ba, ca, ai, bi, ci, ex, ey);
            if (record) {
                if (acc_k != k_old) {
                    if (acc_k >= 0) path.add(acc_k, acc);
                    acc_k = k_old; acc = T(0);
                }
                acc += dist;
            }
            remains -= dist * bv;
            if (k >= 0 && k <= top) continue;
            outcome = k > top ? 2 : 1;
            break;
        }
        if (PATHS && acc_k >= 0) path.add(acc_k, acc);
        if (outcome == 4) {  // budget spent: the walk resumes next iteration
            if (QUEUE) P.paused[out][warp_reserve(P.counts + kListCounts * out, 3)] = slot;
            break;
        }
        // A finished history leaves its slot empty until the next launch, where it is
        // refilled before the walks start: claiming and walking a second photon here
        // would make the whole warp wait on the few lanes whose photon escaped.
        if (outcome == 3) { atomicOr(failure, kHistoryCap); pid = kNone; break; }
        if (outcome == 2) { pid = kNone; break; }
        int kind;
        if (outcome == 1) {
            if (PATHS && k1 == -2) { k1 = -1; init_part = T(0); }
            k = 0;
            z = T(0);
            weight *= __ldg(s.albedo + i + s.nx * j);
            if (weight < eps) { pid = kNone; break; }
            kind = 255;
        } else {
            if (PATHS && k1 == -2) {
                k1 = k;
                init_part = (__ldg(s.zunit + k) - z) * ci;
            }
            const T rtemp = T(rng.next());
            int sp = -1;
            const T* cellp = s.cells + 4 * (i + s.nx * (j + s.ny * k));
            for (int q = 0; q < s.ntypes; ++q)
                if (__ldg(cellp + 1 + q) > rtemp) { sp = q; break; }
            weight *= sp < 0 ? __ldg(s.ssalb_gas + k) : s.ssalb_aer[sp];
            if (weight < eps) { pid = kNone; break; }
            kind = sp + 1;
        }
        ++scatters;
        ++order;
        const int queue = kind == 255 ? kQueueSurface : (kind == 0 ? kQueueGas : kQueueParticle);
        if (QUEUE) P.queue[out][queue][warp_reserve(P.counts + kListCounts * out, queue)] = slot;
        pending = kind;
        event = queue;
        break;
    }

    if (pid == kNone) {
        if (meta.x != kNone || fresh) P.meta(slot) = make_uint4(kNone, 0u, 0u, 0u);
        // An empty slot waits for the next launch: copies still waiting keep it live; while
        // photons remain to claim it is refilled there.
        if (QUEUE && ((P.waiting && P.waiting[slot] > 0u) || may_claim))
            P.vacant[out][warp_reserve(P.counts + kListCounts * out, 4)] = slot;
        return -1;
    }
    // The whole block, direction included (a scattering or a claim changed it; storing it
    // always also keeps every sector of the block fully written).
    if (!P.steps) pol.w = T(steps);
    P.pos(slot) = pos;
    P.dir(slot) = dir;
    P.pol(slot) = pol;
    P.meta(slot) = make_uint4(pid, rng.draw, pack_cell(i, j, pending), pack_layers(k, k1, path.wmin, path.wmax));
    if (P.steps) P.steps[slot] = steps;
    if (P.order) P.order[slot] = order;
    if (PATHS) {
        P.runs[slot] = path.runs;
        P.run_ci[2 * size_t(slot)] = path.ci0;
        P.run_ci[2 * size_t(slot) + 1] = path.ci1;
    }
    if (fresh) {
        if (P.ring_n) P.ring_n[slot] = 0u;
        if (P.vee) P.vee[slot] = vee;
        if (P.lineage) P.lineage[slot] = lineage;
        if (P.matrix) {
            const int nm = s.nmat;
            for (int e = 0; e < nm * nm; ++e) P.matrix[size_t(e) * P.capacity + slot] = (e % (nm + 1) == 0) ? T(1) : T(0);
        }
    }
    return event;
}

// 128-bit tally update (FP32: one vector atomic; FP64: per nonzero element).
__device__ __forceinline__ void quad_add(Quad<float>* p, float x, float y, float z, float w) {
    atomicAdd(reinterpret_cast<float4*>(p), make_float4(x, y, z, w));
}
__device__ __forceinline__ void quad_add(Quad<double>* p, double x, double y, double z, double w) {
    if (x != 0.0) atomicAdd(&p->x, x);
    if (y != 0.0) atomicAdd(&p->y, y);
    if (z != 0.0) atomicAdd(&p->z, z);
    if (w != 0.0) atomicAdd(&p->w, w);
}

__device__ __forceinline__ uint32_t queue_entry(uint32_t* const* queue, uint32_t e, uint32_t ns, uint32_t ng,
                                                bool& surface) {
    surface = e < ns;
    if (surface) return queue[kQueueSurface][e];
    if (e < ns + ng) return queue[kQueueGas][e - ns];
    return queue[kQueueParticle][e - ns - ng];
}

// ----------------------------------------------------------------------------------
// peel: one event per thread, every view.
// ----------------------------------------------------------------------------------
// Peel-off of one event (slot) to every view: the phase matrix, the optical depth along
// each view ray, the register pixel and the tallies (Stokes, layer paths, order records,
// importance ring).
template <typename T, typename TA, int NMAT, bool PATHS, bool BACKWARD>
__device__ __forceinline__ void peel_event(uint32_t slot, bool surface, const SceneView<T>& s,
                                           const T* band, const Controls& ctl, const Divisors& dv, const Pool<T>& P,
                                           TA* __restrict__ banks, const WaveTally& L, uint32_t shard,
                                           uint32_t* __restrict__ failure, uint64_t& visits, uint64_t& updates) {
    const T eps = Tol<T>::eps;
    const int top = s.nz - 1;
    // All records at once, before the test of the entry: one memory latency.
    const uint4 meta = P.meta(slot);
    const Quad<T> pos = P.pos(slot);
    const Quad<T> dir = P.dir(slot);
    const Quad<T> pol = P.pol(slot);
    const uint32_t pid = meta.x;
    if (pid == kNone) { atomicOr(failure, kQueueCorrupt); return; }
    const int i = cell_i(meta.z), j = cell_j(meta.z);
    int k, k1, wmin, wmax;
    unpack_layers(meta.w, k, k1, wmin, wmax);
    const int sp = surface ? -1 : cell_kind(meta.z) - 1;
    const T x = pos.x, y = pos.y, z = pos.z, weight = pos.w;
    const T a = dir.x, b = dir.y, c = dir.z, phi = dir.w;
    const T st[4] = {T(1), pol.x, pol.y, (NMAT > 3 && P.vee) ? P.vee[slot] : T(0)};
    // Backward transport: the history's weight matrix (M11 = 1).
    T M[NMAT][NMAT];
    if (BACKWARD) {
#pragma unroll
        for (int r = 0; r < NMAT; ++r)
#pragma unroll
            for (int q = 0; q < NMAT; ++q) M[r][q] = P.matrix[size_t(r * NMAT + q) * P.capacity + slot];
    }
    const uint32_t round_offset = dv.per_round.div(pid);
    TA* bank = banks + (size_t(round_offset) * L.shards + shard) * L.count;
    Quad<TA>* pixrec = reinterpret_cast<Quad<TA>*>(bank);
    TA* const layer_base = bank + 4 * size_t(L.pixels);
    const T* wander = PATHS ? P.wander + size_t(slot) * s.nz : nullptr;
    const T sin_c = sqrt(fmax(eps, T(1) - c * c));
    T sphi, cphi;
    sincos(phi, &sphi, &cphi);
    T contributed = T(0);  // Stokes-I peel-off of this event, all views
    bool failed = false;
    // Scattering-order diagnostics: the event's history order and its location record
    // (layer 0 = an event on the surface).
    const uint32_t order = P.order ? P.order[slot] : 0u;
    uint32_t location_i = uint32_t(i), location_j = uint32_t(j);
    uint32_t location_layer = (k == 0 && z < eps) ? 0u : uint32_t(k + 1);
    if (BACKWARD && L.orders && P.first) {
        // The sensor of backward transport looks at the history's first event.
        if (order <= 1u) {
            P.first[slot] = location_i | (location_j << 12) | (location_layer << 24);
        } else {
            const uint32_t w = P.first[slot];
            location_i = w & 0xFFFu; location_j = (w >> 12) & 0xFFFu; location_layer = w >> 24;
        }
    }
    // Backward transport registers every view at the injection column.
    uint32_t inject_i = 0, inject_j = 0;
    if (BACKWARD) {
        const uint32_t column = dv.ncol.mod(pid - round_offset * ctl.per_round);
        inject_j = dv.nx.div(column);
        inject_i = column - inject_j * uint32_t(s.nx);
        inject_j = min(inject_j, uint32_t(s.ny - 1));
    }
    for (int ia = 0; ia < s.angles; ++ia) {
        const T vc = s.vc[ia];
        T prob[4] = {T(0), T(0), T(0), T(0)};
        if (surface) {
            if (vc > T(0)) {
                // Forward As S keeps I (= 1); backward M As S0 is the first column of M.
                if (BACKWARD) for (int m = 0; m < NMAT; ++m) prob[m] = M[m][0] * vc * weight;
                else prob[0] = vc * weight;
            }
        } else {
            // cos(phi - phi_view) from the sines and cosines of both azimuths.
            const T cdphi = cphi * s.vcos_phi[ia] + sphi * s.vsin_phi[ia];
            const T cs = c * vc + sin_c * s.vsin[ia] * cdphi;
            const Rot<T> r = NMAT > 1 ? rotation_pre<T>(cs, c, vc, phi, s.vphi[ia], cphi, sphi, s.vcos_phi[ia], s.vsin_phi[ia])
                                      : Rot<T>{T(1), T(0), T(1), T(0)};
            const Phase<T> f = phase<T>(s, sp, cs, NMAT);
            T back[4];
            if (BACKWARD) {
                // M P^T S0: M times the first row of P, (F11, F12 C1, -F12 S1, 0).
                const T row[4] = {f.f11, f.f12 * r.c1, -f.f12 * r.s1, T(0)};
#pragma unroll
                for (int m = 0; m < NMAT; ++m) {
                    T acc = T(0);
#pragma unroll
                    for (int q = 0; q < NMAT; ++q) acc += M[m][q] * row[q];
                    back[m] = acc;
                }
            } else {
                scatter_stokes<T>(f, r, NMAT, st, back);
            }
            for (int m = 0; m < NMAT; ++m) prob[m] = back[m] * weight;
            if (prob[0] < Tol<T>::negligible) for (int m = 0; m < NMAT; ++m) prob[m] = T(0);
        }
        bool finite = true;
        for (int m = 0; m < NMAT; ++m) finite = finite && isfinite(prob[m]);
        if (!finite) { atomicOr(failure, kNonfinite); failed = true; break; }
        if (!(prob[0] > eps)) continue;

        // Detector ray: explicit cell walk below the uniform top, then the prefix.
        const T va = s.va[ia], vb = s.vb[ia];
        T rx = x, ry = y, rz = z;
        if (va * a < T(0)) rx = fmax(T(0), s.xunit - rx);
        if (vb * b < T(0)) ry = fmax(T(0), s.yunit - ry);
        if (vc * c < T(0)) rz = fmax(T(0), __ldg(s.zunit + k) - rz);
        const int is = signbit(va) ? -1 : 1, js = signbit(vb) ? -1 : 1, ks = signbit(vc) ? -1 : 1;
        const T aa = fabs(va), ba = fabs(vb), ca = fabs(vc);
        const T ai = T(1) / fmax(aa, eps), bi = T(1) / fmax(ba, eps), ci = T(1) / fmax(ca, eps);
        const T x_old = rx, y_old = ry, z_old = rz;
        T tau = T(0);
        int ri = i, rj = j, rk = k;
        uint32_t rsteps = 0;
        bool capped = false;
        while (rk >= 0 && rk < top) {
            if (rk >= s.uniform_top) {
                // Uniform layers: one extinction per layer, the same in every cell.
                tau += (rz * __ldg(s.layer_beta + rk) + __ldg(s.tau_above + rk)) * ci;
                ++visits;
                break;
            }
            if (++rsteps > ctl.max_steps) { capped = true; break; }
            // Face by face: view rays cross few band cells, and the rectangle
            // lookup costs more than it skips here (measured on the box cloud).
            const T bv = band_beta<T>(s, band, ri, rj, rk);
            const T dist = advance(s, ri, rj, rk, rx, ry, rz, is, js, ks, aa, ba, ca, ai, bi, ci);
            tau += dist * bv;
            ++visits;
        }
        if (capped) { atomicOr(failure, kDetectorCap); failed = true; break; }
        T height = __ldg(s.zsum + k) + (ks > 0 ? __ldg(s.zunit + k) - z_old : z_old);
        height = __ldg(s.zsum + top) - height;
        const T dxp = aa * height / ca, dyp = ba * height / ca;
        const uint32_t di = uint32_t(((s.xunit - x_old) + dxp) / s.xunit);
        const uint32_t dj = uint32_t(((s.yunit - y_old) + dyp) / s.yunit);
        int pi_ = i + is * int(dv.nx.mod(di));
        pi_ = pi_ < 0 ? pi_ + s.nx : (pi_ >= s.nx ? pi_ - s.nx : pi_);
        int pj_ = j + js * int(dv.ny.mod(dj));
        pj_ = pj_ < 0 ? pj_ + s.ny : (pj_ >= s.ny ? pj_ - s.ny : pj_);
        const uint32_t pixel = BACKWARD ? inject_i + uint32_t(s.nx) * (inject_j + uint32_t(s.ny) * uint32_t(ia))
                                          : uint32_t(pi_ + s.nx * (pj_ + s.ny * ia));
        const T att = exp(-tau);
        const T w = prob[0] * att;
        contributed += P.pixel_weight ? w * __ldg(P.pixel_weight + pixel) : w;
        const T q3 = NMAT > 3 ? prob[3] * att : T(0);
        if (L.orders) {
            const T q1 = NMAT > 1 ? prob[1] * att : T(0), q2 = NMAT > 2 ? prob[2] * att : T(0);
            Quad<TA>* single = reinterpret_cast<Quad<TA>*>(bank + L.orders);
            Quad<TA>* located = single + L.pixels;
            const uint32_t cell = location_i + uint32_t(s.nx) * (location_j + uint32_t(s.ny) * (location_layer + uint32_t(s.nz) * uint32_t(ia)));
            quad_add(located + cell, TA(w), TA(q1), TA(q2), TA(q3));
            if (order == 1u) {
                quad_add(single + pixel, TA(w), TA(q1), TA(q2), TA(q3));
                quad_add(located + L.locations + cell, TA(w), TA(q1), TA(q2), TA(q3));
            }
        }
        quad_add(pixrec + pixel, TA(w), TA(NMAT > 1 ? prob[1] * att : T(0)), TA(NMAT > 2 ? prob[2] * att : T(0)),
                 TA(PATHS ? w : T(0)));
        if (NMAT > 3 && q3 != T(0)) atomicAdd(bank + L.vee + pixel, TA(q3));
        ++updates;
        if (PATHS) {
            TA* const path = layer_base + size_t(pixel) * 2 * L.span;
            TA* const diff = path + L.span;
            // Path pieces, four layers per request: the wander range, the event layer k (the
            // partial view ray) and the first-event layer k1 (the partial descent).
            int lo = k, hi = k;
            if (wmin <= wmax) { lo = min(lo, wmin); hi = max(hi, wmax); }
            if (k1 >= 0) { lo = min(lo, k1); hi = max(hi, k1); }
            const T init_piece = k1 >= 0 ? w * pol.w : T(0);
            for (int g = lo & ~3; g <= hi; g += 4) {
                T v[4];
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const int kk = g + q;
                    T x = (kk >= wmin && kk <= wmax) ? w * wander[kk] : T(0);
                    if (kk == k) x += w * z_old * ci;
                    if (kk == k1) x += init_piece;
                    v[q] = x;
                }
                if (v[0] != T(0) || v[1] != T(0) || v[2] != T(0) || v[3] != T(0)) {
                    quad_add(reinterpret_cast<Quad<TA>*>(path + g), TA(v[0]), TA(v[1]), TA(v[2]), TA(v[3]));
                    ++updates;
                }
            }
            // Straight paths into the difference array: the view ray above the event layer
            // (events in the top layer leave w / mu_view in path element nz instead), the
            // initial descent above the first-event layer, the straight runs; one request
            // per four-layer group touched. Fixed slots (-1 = none) keep them in registers.
            const uint32_t runs = P.runs[slot];
            int at[6];
            T val[6];
            at[0] = k + 1 < s.nz ? k + 1 : -1;
            val[0] = w * ci;
            if (at[0] < 0) { atomicAdd(path + s.nz, TA(val[0])); ++updates; }
            at[1] = k1 >= 0 ? k1 + 1 : 0;
            val[1] = w * s.inv_mu0;
#pragma unroll
            for (int r = 0; r < 2; ++r) {
                const uint32_t lh = (runs >> (16 * r)) & 0xFFFFu;
                const bool run = (lh & 0xFFu) != 0xFFu;
                const T v = run ? w * P.run_ci[2 * size_t(slot) + r] : T(0);
                at[2 + 2 * r] = run ? int(lh & 0xFFu) : -1;
                at[3 + 2 * r] = run ? int(lh >> 8) + 1 : -1;
                val[2 + 2 * r] = v;
                val[3 + 2 * r] = -v;
            }
            uint32_t done = 0u;
#pragma unroll
            for (int q = 0; q < 6; ++q) {
                if (at[q] < 0 || ((done >> q) & 1u)) continue;
                const int g = at[q] & ~3;
                T v0 = T(0), v1 = T(0), v2 = T(0), v3 = T(0);
#pragma unroll
                for (int r = q; r < 6; ++r) {
                    if (at[r] < 0 || ((done >> r) & 1u) || (at[r] & ~3) != g) continue;
                    const int j = at[r] - g;
                    v0 += j == 0 ? val[r] : T(0);
                    v1 += j == 1 ? val[r] : T(0);
                    v2 += j == 2 ? val[r] : T(0);
                    v3 += j == 3 ? val[r] : T(0);
                    done |= 1u << r;
                }
                quad_add(reinterpret_cast<Quad<TA>*>(diff + g), TA(v0), TA(v1), TA(v2), TA(v3));
                ++updates;
            }
        }
    }
    if (P.ring_n && !failed) {
        // Importance tally: this event enters the ring, and its contribution is credited,
        // per unit weight, to every event of the ring (itself included).
        const uint32_t cells = uint32_t(s.nx) * uint32_t(s.ny) * uint32_t(s.nz);
        const uint32_t cell = uint32_t(i) + uint32_t(s.nx) * (uint32_t(j) + uint32_t(s.ny) * uint32_t(k));
        const uint32_t n = P.ring_n[slot];
        uint32_t* rc = P.ring_cell + size_t(slot) * kRing;
        T* ri = P.ring_inv + size_t(slot) * kRing;
        rc[n % kRing] = cell;
        ri[n % kRing] = T(1) / weight;
        P.ring_n[slot] = n + 1;
        atomicAdd(P.importance + cells + cell, 1.0);
        if (contributed != T(0)) {
            const uint32_t live = min(n + 1, uint32_t(kRing));
            for (uint32_t q = 0; q < live; ++q) atomicAdd(P.importance + rc[q], double(contributed * ri[q]));
        }
    }
}

template <typename T, typename TA, int NMAT, bool PATHS, bool BACKWARD>
__device__ __forceinline__ void peel_phase(const SceneView<T>& s, const T* band, const Controls& ctl,
                                           const Divisors& dv, const Pool<T>& P, TA* __restrict__ banks,
                                           const WaveTally& L, uint32_t b, uint32_t* __restrict__ failure,
                                           unsigned long long* __restrict__ counters, uint32_t block = blockIdx.x,
                                           uint32_t blocks = gridDim.x) {
    const uint32_t* c = P.counts + kListCounts * b;
    const uint32_t ns = c[0], ng = c[1], np = c[2];
    const uint32_t total = ns + ng + np;
    const uint32_t shard = ((block * blockDim.x + threadIdx.x) >> 5) % L.shards;
    uint64_t visits = 0, updates = 0;

    for (uint32_t e = block * blockDim.x + threadIdx.x; e < total; e += blocks * blockDim.x) {
        bool surface;
        const uint32_t slot = queue_entry(P.queue[b], e, ns, ng, surface);
        if (slot >= P.capacity) { atomicOr(failure, kQueueCorrupt); continue; }
        peel_event<T, TA, NMAT, PATHS, BACKWARD>(slot, surface, s, band, ctl, dv, P, banks, L, shard, failure, visits,
                                                 updates);
    }
    const unsigned long long totals[2] = {visits, updates};
    unsigned long long* const targets[2] = {counters + 2, counters + 3};
    block_add<2>(totals, targets);
}

// FP32: four blocks of 256 per SM (64 registers; +2.7 % on the layered cloud over three
// blocks at 77 registers, the box cloud unchanged). FP64 stays at three: at 64 registers its
// peel-off spills 200-400 bytes per thread.
template <typename T, typename TA, int NMAT, bool PATHS, bool BACKWARD>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? 4 : 3)
wf_peel(SceneView<T> s, Controls ctl, Divisors dv, Pool<T> P, TA* __restrict__ banks, WaveTally L, uint32_t b,
        uint32_t* __restrict__ failure, unsigned long long* __restrict__ counters) {
    extern __shared__ __align__(16) unsigned char staged[];
    const T* band = stage_band<T>(s, staged, failure);
    peel_phase<T, TA, NMAT, PATHS, BACKWARD>(s, band, ctl, dv, P, banks, L, b, failure, counters);
}

// ----------------------------------------------------------------------------------
// scatter: new direction (and Stokes vector) for every queued event.
// ----------------------------------------------------------------------------------
// Guided transport: detector directional importance sampling (DDIS) and Russian roulette,
// the unbiased variance reduction of Buras & Mayer (2011), "Efficient unbiased variance
// reduction techniques for Monte Carlo simulations of radiative transfer in cloudy
// atmospheres: The solution", JQSRT 112, 434-447. At a particle scatter, with probability
// epsilon the new direction is drawn about a detector direction (a view picked uniformly)
// from the particle's own cosine proposal with a uniform azimuth, otherwise by the analog
// polarized sampler; the weight is then multiplied by p_analog / q with
// q = (1 - epsilon) p_analog + epsilon p_detector, so every estimate keeps its analog
// expectation. After every scatter a photon lighter than the cell's roulette weight W
// survives with probability weight / W, at weight W.

// Density per unit cosine of the analog cosine proposal of species sp: the bound CDF is
// interpolated linearly in cosine, so the density is constant between table nodes.
template <typename T>
__device__ __forceinline__ T proposal_density(const SceneView<T>& s, int sp, T cs) {
    const int n = s.lut_n[sp];
    const T* __restrict__ cosv = s.lut_cos[sp];
    const T* __restrict__ cdf = s.lut_cdf[sp];
    int lo = lut_bracket(cosv, n, cs);
    if (lo > n - 2) lo = n - 2;
    return (__ldg(cdf + lo + 1) - __ldg(cdf + lo)) / (__ldg(cosv + lo + 1) - __ldg(cosv + lo));
}

// p_analog / q for a particle scatter into (a, b, c) at scattering cosine cs; s0 is the
// scattered intensity of the unit incident Stokes vector (the acceptance pdf).
template <typename T, int NMAT>
__device__ __forceinline__ T ddis_factor(const SceneView<T>& s, const Guide<T>& g, int sp, T cs, T s0, T a, T b, T c) {
    const Phase<T> f = particle<T>(s, sp, cs, NMAT);
    const T bound = f.f11 + fabs(f.f12);
    const T p_an = bound > T(0) ? proposal_density<T>(s, sp, cs) * (s0 / bound) / s.znorm[sp] : T(0);
    T p_det = T(0);
    for (int v = 0; v < s.angles; ++v) {
        const T cv = a * s.va[v] + b * s.vb[v] + c * s.vc[v];
        p_det += proposal_density<T>(s, sp, fmin(T(1), fmax(T(-1), cv)));
    }
    p_det /= T(s.angles);
    const T q = (T(1) - g.epsilon) * p_an + g.epsilon * p_det;
    return q > T(0) ? p_an / q : T(0);
}

// Scattering of one event (slot): the new direction (Lambert, polarized sampling or the
// guided detector branch), the Stokes or weight-matrix update, roulette and the next free
// path. Returns false when the photon ends here. With `handoff` the slot's new records go
// there (for a walk in the same thread) instead of to memory; a photon that ends is still
// marked empty in memory.
template <typename T, int NMAT, bool BACKWARD>
__device__ __forceinline__ bool scatter_event(uint32_t slot, bool surface, const SceneView<T>& s,
                                              const Controls& ctl, const Divisors& dv, const Pool<T>& P,
                                              const Guide<T>& g, uint32_t* __restrict__ failure,
                                              SlotState<T>* handoff = nullptr) {
    const T eps = Tol<T>::eps;
    const T pi = pi_v<T>();
    // All records at once, before the test of the entry: one memory latency.
    uint4 meta = P.meta(slot);
    Quad<T> pos = P.pos(slot);
    const Quad<T> dir0 = P.dir(slot);
    Quad<T> pol = P.pol(slot);
    const uint32_t pid = meta.x;
    auto ended = [&]() {
        P.meta(slot) = make_uint4(kNone, 0u, 0u, 0u);
        if (handoff) handoff->meta = make_uint4(kNone, 0u, 0u, 0u);
        return false;
    };
    if (pid == kNone) {
        atomicOr(failure, kQueueCorrupt);
        if (handoff) handoff->meta = meta;
        return false;
    }
    const uint32_t ro = dv.per_round.div(pid);
    DrawStream rng;
    rng.init(pid - ro * ctl.per_round, ctl.first_round + ro, ctl.seed, meta.y, P.lineage ? P.lineage[slot] : 0u);
    const T a0 = dir0.x, b0 = dir0.y, c0 = dir0.z;
    T a, b, c, phi_out, q = T(0), u = T(0), v = T(0);
    // Backward transport: the weight matrix (M11 = 1), updated by M P^T (M As at the
    // surface) and renormalized by its M11.
    T M[NMAT][NMAT];
    if (BACKWARD) {
#pragma unroll
        for (int r = 0; r < NMAT; ++r)
#pragma unroll
            for (int col = 0; col < NMAT; ++col) M[r][col] = P.matrix[size_t(r * NMAT + col) * P.capacity + slot];
    }
    const int ci = cell_i(meta.z), cj = cell_j(meta.z), ck = int(meta.w & 0xFF) - 1;
    T roulette = g.roulette;
    if (g.scale) roulette *= __ldg(g.scale + ci + s.nx * (cj + s.ny * ck));
    if (surface) {
        const T Pd = T(rng.next()), U = T(rng.next());
        if (roulette > T(0) && pos.w < roulette) {
            if (T(rng.next()) * roulette < pos.w) pos.w = roulette;
            else return ended();
        }
        const T mu = sqrt(Pd);
        phi_out = T(2) * pi * U;
        const T sine = sqrt(fmax(T(0), T(1) - mu * mu));
        T sp, cp;
        sincos(phi_out, &sp, &cp);
        a = sine * cp; b = sine * sp; c = fabs(mu);
        if (BACKWARD) {
            // M As keeps the first column of M; then M / M11.
            const T m11 = M[0][0];
#pragma unroll
            for (int r = 0; r < NMAT; ++r) {
#pragma unroll
                for (int col = 1; col < NMAT; ++col) M[r][col] = T(0);
                M[r][0] = M[r][0] / m11;
            }
        }
    } else {
        const int sp = cell_kind(meta.z) - 1;
        const T phi = dir0.w;
        T st[4] = {T(1), pol.x, pol.y, (NMAT > 3 && P.vee) ? P.vee[slot] : T(0)};
        T cos_out, dphi, cos_sca;
        const bool guided = sp >= 0 && g.epsilon > T(0) && pos.w < g.cap;
        if (guided && T(rng.next()) < g.epsilon) {
            // Detector branch: a view, a cosine about it from the proposal, an azimuth.
            const int v = min(int(T(rng.next()) * T(s.angles)), s.angles - 1);
            const T cd = sample_cdf<T>(s, sp, T(rng.next()));
            const T psi = T(2) * pi * T(rng.next());
            const T dx = s.va[v], dy = s.vb[v], dz = s.vc[v];
            const T h = sqrt(dx * dx + dy * dy);
            const bool tilted = h > T(1e-12);
            const T e1x = tilted ? -dy / h : T(1), e1y = tilted ? dx / h : T(0);
            const T e2x = -dz * e1y, e2y = dz * e1x, e2z = dx * e1y - dy * e1x;
            const T sd = sqrt(fmax(T(0), T(1) - cd * cd));
            T spsi, cpsi;
            sincos(psi, &spsi, &cpsi);
            const T wx = cd * dx + sd * (cpsi * e1x + spsi * e2x);
            const T wy = cd * dy + sd * (cpsi * e1y + spsi * e2y);
            const T wz = cd * dz + sd * spsi * e2z;
            cos_out = fmin(T(1), fmax(T(-1), wz));
            phi_out = atan2(wy, wx);
            const T so = sqrt(fmax(T(0), T(1) - cos_out * cos_out));
            T sp_, cp_;
            sincos(phi_out, &sp_, &cp_);
            cos_sca = fmin(T(1), fmax(T(-1), a0 * (cp_ * so) + b0 * (sp_ * so) + c0 * cos_out));
        } else {
            if (!sample_direction<T>(s, sp, NMAT, st, c0, rng, cos_out, dphi, cos_sca, BACKWARD ? T(1) : T(-1))) {
                atomicOr(failure, kSamplingCap);
                return ended();
            }
            phi_out = phi + dphi;
        }
        const Rot<T> r = NMAT > 1 ? rotation<T>(cos_sca, c0, cos_out, phi, phi_out) : Rot<T>{T(1), T(0), T(1), T(0)};
        const Phase<T> f = phase<T>(s, sp, cos_sca, NMAT);
        T out[4] = {T(0), T(0), T(0), T(0)};
        if (BACKWARD) {
            // M = M P^T; the sampling vector is (M11, M12, -M13, M14).
            T Pm[4][4];
            phase_matrix<T>(f, r, NMAT, Pm);
            T next[NMAT][NMAT];
#pragma unroll
            for (int row = 0; row < NMAT; ++row)
#pragma unroll
                for (int col = 0; col < NMAT; ++col) {
                    T acc = T(0);
#pragma unroll
                    for (int k2 = 0; k2 < NMAT; ++k2) acc += M[row][k2] * Pm[col][k2];
                    next[row][col] = acc;
                }
            const T m11 = next[0][0];
#pragma unroll
            for (int row = 0; row < NMAT; ++row)
#pragma unroll
                for (int col = 0; col < NMAT; ++col) M[row][col] = next[row][col] / m11;
            out[0] = next[0][0];
            if (NMAT > 1) { out[1] = next[0][1]; out[2] = -next[0][2]; }
            if (NMAT > 3) out[3] = next[0][3];
        } else {
            scatter_stokes<T>(f, r, NMAT, st, out);
        }
        // S / S(1): I becomes 1 (NaN when S(1) is 0 or not finite).
        const T s0 = out[0];
        const T one = s0 / s0;
        bool ok = isfinite(one);
        if (NMAT > 1) {
            q = out[1] / s0; u = out[2] / s0;
            if (NMAT > 3) v = out[3] / s0;
            ok = ok && isfinite(q) && isfinite(u) && isfinite(v) && sqrt(q * q + u * u + v * v) <= one + T(1e-2);
        }
        if (!ok) { atomicOr(failure, kInvalidStokes); return ended(); }
        const T so = sqrt(fmax(T(0), T(1) - cos_out * cos_out));
        T spo, cpo;
        sincos(phi_out, &spo, &cpo);
        a = cpo * so; b = spo * so; c = cos_out;
        if (guided) pos.w *= ddis_factor<T, NMAT>(s, g, sp, cos_sca, s0, a, b, c);
        if (roulette > T(0) && pos.w < roulette) {
            if (T(rng.next()) * roulette < pos.w) pos.w = roulette;
            else return ended();
        }
    }
    if (a * a0 < T(0)) pos.x = fmax(T(0), s.xunit - pos.x);
    if (b * b0 < T(0)) pos.y = fmax(T(0), s.yunit - pos.y);
    if (c * c0 < T(0)) {
        const int k = int(meta.w & 0xFF) - 1;
        pos.z = fmax(T(0), __ldg(s.zunit + k) - pos.z);
    }
    pol.x = q; pol.y = u;
    if (!surface && g.split > T(0) && P.waiting && roulette > T(0) && pos.w > g.split * roulette) {
        // Splitting: n copies of weight / n, n - 1 of them left waiting in this slot, each
        // with its own stream (drawn before this history's next free path).
        const uint32_t held = P.waiting[slot];
        const int n = min(min(int(pos.w / roulette), kSplitMax), 1 + kSplitStack - int(held));
        if (n >= 2) {
            pos.w = pos.w / T(n);
            const uint32_t lineage = P.lineage[slot];
            const uint32_t order = P.order ? P.order[slot] : 0u;
            const Quad<T> dir_out{a, b, c, phi_out};
            const Quad<T> pol_out{q, u, v, pol.w};
            for (int copy = 1; copy < n; ++copy) {
                const size_t entry = size_t(slot) * kSplitStack + held + uint32_t(copy) - 1u;
                SplitCopy<T>& cp = P.copies[entry];
                cp.meta = make_uint4(pid, split_lineage(lineage, rng.draw, uint32_t(copy)), meta.z, meta.w);
                cp.pos = pos;
                cp.dir = dir_out;
                cp.pol = pol_out;
                if (P.copy_order) P.copy_order[entry] = order;
            }
            P.waiting[slot] = held + uint32_t(n) - 1u;
        }
    }
    if (NMAT > 3 && P.vee) P.vee[slot] = v;
    if (BACKWARD) {
#pragma unroll
        for (int r = 0; r < NMAT; ++r)
#pragma unroll
            for (int col = 0; col < NMAT; ++col) P.matrix[size_t(r * NMAT + col) * P.capacity + slot] = M[r][col];
    }
    if (!surface) pol.z = -log(fmax(T(rng.next()), eps));
    meta.y = rng.draw;
    const Quad<T> turned{a, b, c, phi_out};
    if (handoff) {
        *handoff = SlotState<T>{meta, pos, turned, pol};
        return true;
    }
    P.pos(slot) = pos;
    P.dir(slot) = turned;
    P.pol(slot) = pol;
    P.meta(slot) = meta;
    return true;
}

// ----------------------------------------------------------------------------------
// step: one wavefront iteration's scattering and walks, reading the work lists of buffer
// `cur` and filing every slot in those of buffer 1 - cur. Each queued event is scattered
// and its photon walks on to its next event in the same thread, with no launch in between
// (the scattered records pass to the walk within the thread, and the walk stores the
// slot's block once); paused photons resume their walks; vacant slots take a waiting
// split copy or the next photon of the round group and walk it. One thread per list
// entry: the lists hold at most one entry per slot.
// ----------------------------------------------------------------------------------
template <typename T, int NMAT, bool PATHS, bool BACKWARD, bool SMEM_HANDOFF = false>
__device__ __forceinline__ void step_phase(const SceneView<T>& s, const T* band, const Controls& ctl,
                                           const Divisors& dv, const Pool<T>& P, const Guide<T>& g, uint32_t walk,
                                           uint32_t cur, uint32_t* __restrict__ failure,
                                           unsigned long long* __restrict__ counters, uint32_t block = blockIdx.x,
                                           uint32_t blocks = gridDim.x) {
    const uint32_t* c = P.counts + kListCounts * cur;
    const uint32_t ns = c[0], ng = c[1], np = c[2], held = c[3], vacant = c[4];
    const uint32_t events = ns + ng + np, total = events + held + vacant;
    const uint32_t out = cur ^ 1u;
    uint64_t scatters = 0, visits = 0;
    // Once every photon of the group is claimed (the counter only grows), vacant slots stop
    // at once: one read per block instead of one per lane on a single address.
    __shared__ uint32_t claims_open;
    if (threadIdx.x == 0) claims_open = *reinterpret_cast<volatile uint32_t*>(P.counts + kClaimCount) < ctl.count;
    __syncthreads();
    const bool may_claim = claims_open != 0u;

    // The scattered records pass to the walk through a per-thread slot in shared memory
    // (SMEM_HANDOFF; 1 % faster on the box cloud than the thread's stack, whose misses in L1
    // go to L2) or on the thread's stack (the multi-scene kernel, whose staged bands leave no
    // room). 80-byte stride in FP32: the 16-byte accesses of a quarter warp fall in distinct
    // banks; 128 in FP64 for the 32-byte alignment of its records.
    constexpr int kHandStride = sizeof(T) == 4 ? 80 : 128;
    __shared__ __align__(32) unsigned char hand[SMEM_HANDOFF ? 256 * kHandStride : 16];
    SlotState<T> local_state;
    SlotState<T>& state = SMEM_HANDOFF ? *reinterpret_cast<SlotState<T>*>(hand + threadIdx.x * kHandStride) : local_state;
    for (uint32_t e = block * blockDim.x + threadIdx.x; e < total; e += blocks * blockDim.x) {
        uint32_t slot;
        const bool scattered = e < events;
        if (scattered) {
            bool surface;
            slot = queue_entry(P.queue[cur], e, ns, ng, surface);
            if (slot >= P.capacity) { atomicOr(failure, kQueueCorrupt); continue; }
            // The new records go to the walk through the handoff (it may also leave the slot vacant).
            scatter_event<T, NMAT, BACKWARD>(slot, surface, s, ctl, dv, P, g, failure, &state);
        } else {
            slot = e < events + held ? P.paused[cur][e - events] : P.vacant[cur][e - events - held];
            if (slot >= P.capacity) { atomicOr(failure, kQueueCorrupt); continue; }
        }
        transit_slot<T, PATHS, true>(slot, s, band, ctl, dv, P, walk, may_claim, out, failure, scatters, visits,
                                     scattered ? &state : nullptr);
    }
    const unsigned long long totals[2] = {scatters, visits};
    unsigned long long* const targets[2] = {counters + 0, counters + 1};
    block_add<2>(totals, targets);
}

template <typename T, int NMAT, bool PATHS, bool BACKWARD>
__global__ void __launch_bounds__(256, MONKI_STEP_BLOCKS)
wf_step(SceneView<T> s, Controls ctl, Divisors dv, Pool<T> P, Guide<T> g, uint32_t walk, uint32_t cur,
        uint32_t* __restrict__ failure, unsigned long long* __restrict__ counters) {
    extern __shared__ __align__(16) unsigned char staged[];
    const T* band = stage_band<T>(s, staged, failure);
    step_phase<T, NMAT, PATHS, BACKWARD, true>(s, band, ctl, dv, P, g, walk, cur, failure, counters);
}

// The same iteration in two launches, for scenes with layer paths, whose walks and
// scatterings together need more registers than one kernel has without spilling: the walks
// of every slot in slot order (transit), then, after the peel-off, the scatterings of the
// queued events (scatter). Both file slots in the work lists of buffer `out` like the step.
template <typename T, bool PATHS>
__global__ void __launch_bounds__(256, 4)
wf_transit(SceneView<T> s, Controls ctl, Divisors dv, Pool<T> P, uint32_t walk, uint32_t out,
           uint32_t* __restrict__ failure, unsigned long long* __restrict__ counters) {
    extern __shared__ __align__(16) unsigned char staged[];
    const T* band = stage_band<T>(s, staged, failure);
    uint64_t scatters = 0, visits = 0;
    __shared__ uint32_t claims_open;
    if (threadIdx.x == 0) claims_open = *reinterpret_cast<volatile uint32_t*>(P.counts + kClaimCount) < ctl.count;
    __syncthreads();
    const bool may_claim = claims_open != 0u;
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < P.capacity; slot += gridDim.x * blockDim.x)
        transit_slot<T, PATHS, true>(slot, s, band, ctl, dv, P, walk, may_claim, out, failure, scatters, visits);
    const unsigned long long totals[2] = {scatters, visits};
    unsigned long long* const targets[2] = {counters + 0, counters + 1};
    block_add<2>(totals, targets);
}

template <typename T, int NMAT, bool BACKWARD>
__global__ void __launch_bounds__(256, 4)
wf_scatter(SceneView<T> s, Controls ctl, Divisors dv, Pool<T> P, Guide<T> g, uint32_t b,
           uint32_t* __restrict__ failure) {
    const uint32_t* c = P.counts + kListCounts * b;
    const uint32_t ns = c[0], ng = c[1], total = c[0] + c[1] + c[2];
    for (uint32_t e = blockIdx.x * blockDim.x + threadIdx.x; e < total; e += gridDim.x * blockDim.x) {
        bool surface;
        const uint32_t slot = queue_entry(P.queue[b], e, ns, ng, surface);
        if (slot >= P.capacity) { atomicOr(failure, kQueueCorrupt); continue; }
        scatter_event<T, NMAT, BACKWARD>(slot, surface, s, ctl, dv, P, g, failure);
    }
}

// Start of a round group: every slot empty and listed vacant in buffer 0, no claims yet.
template <typename T>
__global__ void wf_reset(Pool<T> P) {
    const uint32_t stride = gridDim.x * blockDim.x;
    for (uint32_t slot = blockIdx.x * blockDim.x + threadIdx.x; slot < P.capacity; slot += stride) {
        P.meta(slot) = make_uint4(kNone, 0u, 0u, 0u);
        P.vacant[0][slot] = slot;
        if (P.waiting) P.waiting[slot] = 0u;
    }
    if (blockIdx.x == 0 && threadIdx.x < kCountWords)
        P.counts[threadIdx.x] = threadIdx.x == 4 ? P.capacity : 0u;
}

// ----------------------------------------------------------------------------------
// tail: the end of a round group in one launch. Once every photon is claimed and few
// remain, a wavefront iteration has little work and its three launches cost more than
// the work; the longest cloud histories need a hundred or more such iterations. Here each
// thread takes live slots one at a time (reserved together with the other idle lanes of
// its warp) and runs each photon to its end: walk, peel-off and scattering, event after
// event, through the same slot functions as the wavefront kernels.
// ----------------------------------------------------------------------------------
// pending = true: the events queued in buffer b, peeled but not yet scattered (the fused
// step scatters them in the next iteration), are scattered first; pending = false: every
// other live slot (paused walks, waiting split copies).
template <typename T, int NMAT, bool PATHS, bool BACKWARD>
__global__ void __launch_bounds__(256, 2)
wf_tail(SceneView<T> s, Controls ctl, Divisors dv, Pool<T> P, T* __restrict__ banks, WaveTally L, Guide<T> g,
        uint32_t b, bool pending, uint32_t* __restrict__ failure, unsigned long long* __restrict__ counters,
        uint32_t* __restrict__ next) {
    extern __shared__ __align__(16) unsigned char staged[];
    const T* band = stage_band<T>(s, staged, failure);
    const uint32_t shard = ((blockIdx.x * blockDim.x + threadIdx.x) >> 5) % L.shards;
    const uint32_t* c = P.counts + kListCounts * b;
    const uint32_t ns = c[0], ng = c[1], events = c[0] + c[1] + c[2];
    uint64_t scatters = 0, visits = 0, detector = 0, updates = 0;
    for (;;) {
        const uint32_t n = warp_reserve(next);
        uint32_t slot = n;
        if (pending) {
            if (n >= events) break;
            bool surface;
            slot = queue_entry(P.queue[b], n, ns, ng, surface);
            if (slot >= P.capacity) { atomicOr(failure, kQueueCorrupt); continue; }
            if (!scatter_event<T, NMAT, BACKWARD>(slot, surface, s, ctl, dv, P, g, failure) &&
                !(P.waiting && P.waiting[slot] > 0u))
                continue;
        } else {
            if (slot >= P.capacity) break;
            if (P.meta(slot).x == kNone && !(P.waiting && P.waiting[slot] > 0u)) continue;
        }
        // No step budget: the walk pauses only at the history step cap, which ends it.
        for (;;) {
            const int queue = transit_slot<T, PATHS, false>(slot, s, band, ctl, dv, P, 0xFFFFFFFFu, false, 0u, failure,
                                                             scatters, visits);
            if (queue < 0) {
                if (P.waiting && P.waiting[slot] > 0u) continue;  // its split copies next
                break;
            }
            const bool surface = queue == kQueueSurface;
            peel_event<T, T, NMAT, PATHS, BACKWARD>(slot, surface, s, band, ctl, dv, P, banks, L, shard, failure,
                                                    detector, updates);
            if (!scatter_event<T, NMAT, BACKWARD>(slot, surface, s, ctl, dv, P, g, failure) &&
                !(P.waiting && P.waiting[slot] > 0u))
                break;
        }
    }
    const unsigned long long totals[4] = {scatters, visits, detector, updates};
    unsigned long long* const targets[4] = {counters + 0, counters + 1, counters + 2, counters + 3};
    block_add<4>(totals, targets);
}

// ----------------------------------------------------------------------------------
// FP64 flush of the wavefront tallies into RawTallies order, with the prefix sums of
// the straight initial-descent and detector-ray layers. info: zunit[nz] (km),
// 1/|mu0|, then 1/mu per view, then mu0/mu per view.
// ----------------------------------------------------------------------------------
template <typename TA>
__global__ void wf_flush(const TA* __restrict__ banks, WaveTally L, int nmat, int nx, int ny, int nz, int angles,
                         const double* __restrict__ info, uint32_t rounds, uint32_t out_count, bool paths,
                         double* __restrict__ out) {
    const uint32_t pixels = L.pixels;
    const uint32_t stokes_out = uint32_t(nmat) * pixels;
    const uint64_t total = uint64_t(out_count) * rounds;
    const double* zunit = info;
    const double inv_mu0 = info[nz];
    const double* inv_mu = info + nz + 1;
    const double* mu0mu = info + nz + 1 + angles;
    for (uint64_t e = blockIdx.x * uint64_t(blockDim.x) + threadIdx.x; e < total; e += uint64_t(gridDim.x) * blockDim.x) {
        const uint32_t r = uint32_t(e / out_count);
        const uint32_t o = uint32_t(e % out_count);
        const TA* base = banks + size_t(r) * L.shards * L.count;
        auto sum = [&](size_t index) {
            double acc = 0.0;
            for (uint32_t sh = 0; sh < L.shards; ++sh) acc += double(base[size_t(sh) * L.count + index]);
            return acc;
        };
        double value;
        if (o < stokes_out) {
            const uint32_t m = o % uint32_t(nmat);
            const uint32_t pixel = o / uint32_t(nmat);
            const uint32_t ia = pixel / uint32_t(nx * ny);
            value = (m < 3 ? sum(size_t(pixel) * 4 + m) : sum(size_t(L.vee) + pixel)) * mu0mu[ia];
        } else if (paths && o < stokes_out + pixels * uint32_t(nz)) {
            const uint32_t q = o - stokes_out;  // i + nx * (j + ny * (k + nz * ia))
            const uint32_t i = q % nx;
            uint32_t t = q / nx;
            const uint32_t j = t % ny; t /= ny;
            const int k = int(t % nz);
            const uint32_t ia = t / nz;
            const uint32_t pixel = i + nx * (j + ny * ia);
            const size_t path = 4 * size_t(pixels) + size_t(pixel) * 2 * L.span;
            const size_t diff = path + L.span;
            value = sum(path + size_t(k));
            double straight = 0.0;
            for (int s = 0; s <= k; ++s) straight += sum(diff + size_t(s));
            // View rays cross no part of the top layer: take out every view-ray weight
            // (the pixel's detected weight, except that of events in the top layer).
            if (k == nz - 1) straight -= inv_mu[ia] * sum(size_t(pixel) * 4 + 3) - sum(path + size_t(nz));
            value += zunit[k] * straight;
        } else if (!L.orders || o < stokes_out + (paths ? pixels * uint32_t(nz + 1) : 0u)) {
            const uint32_t pixel = o - stokes_out - pixels * uint32_t(nz);
            value = sum(size_t(pixel) * 4 + 3);
        } else {
            // Order diagnostics: single-scattering Stokes, then the location records (all
            // orders, then single scattering), each times mu0/mu of its view.
            const uint32_t q = o - stokes_out - (paths ? pixels * uint32_t(nz + 1) : 0u);
            const uint32_t m = q % uint32_t(nmat);
            const uint32_t record = q / uint32_t(nmat);
            const uint32_t ia = record < pixels ? record / uint32_t(nx * ny)
                                                : ((record - pixels) % L.locations) / uint32_t(nx * ny * nz);
            value = sum(size_t(L.orders) + size_t(record) * 4 + m) * mu0mu[ia];
        }
        out[e] = value;
    }
}

}  // namespace monki
