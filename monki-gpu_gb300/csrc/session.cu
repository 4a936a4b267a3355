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

#include "host_tables.h"
#include "tail.h"
#include "statistics.cuh"
#include "wavefront.cuh"

namespace monki {
namespace {

using namespace host;

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
    uint32_t held = 0;                // rounds of s.out run by monki_cuda_run_held
    uint32_t held_next = 0;           // the next of them to fold
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
    const size_t block = n * kRecordBytes<T>;
    const size_t ring = s.cfg.importance ? n * kRing : 0;
    const size_t parts[] = {block, s.prep.paths ? n * sizeof(uint32_t) : 0,
                            n * nz * sizeof(T), n * sizeof(uint32_t), 2 * n * sizeof(T),
                            10 * n * sizeof(uint32_t), kCountWords * sizeof(uint32_t),
                            ring * sizeof(uint32_t), ring * sizeof(T), s.cfg.importance ? n * sizeof(uint32_t) : 0,
                            s.cfg.orders ? n * sizeof(uint32_t) : 0,
                            (s.prep.nmat == 4 && !s.prep.backward) ? n * sizeof(T) : 0,
                            s.prep.backward ? size_t(s.prep.nmat) * s.prep.nmat * n * sizeof(T) : 0,
                            (s.prep.backward && s.cfg.orders) ? n * sizeof(uint32_t) : 0,
                            s.cfg.split > 0.0 ? n * sizeof(uint32_t) : 0,
                            s.cfg.split > 0.0 ? n * kSplitStack * sizeof(SplitCopy<T>) : 0,
                            (s.cfg.split > 0.0 && s.cfg.orders) ? n * kSplitStack * sizeof(uint32_t) : 0,
                            s.cfg.split > 0.0 ? n * sizeof(uint32_t) : 0};
    size_t bytes = 0;
    for (size_t part : parts) bytes += align_up(part, 256);
    check(cudaMalloc(&s.pool_memory, bytes), "cudaMalloc(pool)");
    char* p = static_cast<char*>(s.pool_memory);
    auto take = [&](size_t b) { char* q = p; p += align_up(b, 256); return q; };
    Pool<T> P{};
    P.capacity = uint32_t(n);
    P.records = reinterpret_cast<unsigned char*>(take(block));
    // Scenes without layer paths keep each walk's step count in its record block.
    if (s.prep.paths) P.steps = reinterpret_cast<uint32_t*>(take(n * sizeof(uint32_t)));
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
        if (s.cfg.orders) P.copy_order = reinterpret_cast<uint32_t*>(take(n * kSplitStack * sizeof(uint32_t)));
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
// Opt a kernel into kBandMaxBytes of dynamic shared memory, once per kernel and device.
void allow_band(const void* fn) {
    static std::mutex lock;
    static std::vector<std::pair<const void*, int>> done;
    int device = 0;
    check(cudaGetDevice(&device), "cudaGetDevice");
    std::lock_guard<std::mutex> guard(lock);
    const std::pair<const void*, int> key{fn, device};
    if (std::find(done.begin(), done.end(), key) != done.end()) return;
    check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kBandMaxBytes)),
          "shared memory attribute");
    done.push_back(key);
}

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
        // A staged band may take all of kBandMaxBytes beside the kernel's own static shared
        // memory, past the 48 KB a launch gets without opting in (set once per kernel).
        if (smem) allow_band(fn);
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
    if (!c.per_round || !c.rounds || c.rounds > s.round_capacity || !c.max_steps || c.max_steps > kMaxHistorySteps ||
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

// Add rounds first .. first + rounds - 1 of s.out to the device accumulators (FP64, rounds in
// order) and write their per-round spatial sums of the normalized Stokes tallies to the host.
void accumulate(Session& s, uint32_t first, uint32_t rounds, double photons_per_column, double* history) {
    const StatsLayout L = statistics_layout(s);
    if (!s.stats) {
        check(cudaMalloc(&s.stats, L.count * sizeof(double)), "cudaMalloc(statistics)");
        check(cudaMemsetAsync(s.stats, 0, L.count * sizeof(double), s.stream), "memset(statistics)");
        check(cudaMalloc(&s.history, size_t(s.round_capacity) * s.prep.nmat * sizeof(double)), "cudaMalloc(history)");
    }
    const uint32_t elements = L.stokes + L.paths + L.weights;
    const int grid = int(std::min<uint32_t>((elements + 255) / 256, 8192));
    // Paths read the weight means of the previous groups, so the weights update second.
    const double* out = s.out + size_t(first) * s.layout.count;
    stats_update<<<grid, 256, 0, s.stream>>>(out, uint32_t(s.layout.count), rounds, uint32_t(s.stats_rounds), L,
                                            photons_per_column, s.stats, 0);
    if (L.weights)
        stats_update<<<grid, 256, 0, s.stream>>>(out, uint32_t(s.layout.count), rounds, uint32_t(s.stats_rounds), L,
                                                photons_per_column, s.stats, 1);
    round_sums<<<dim3(rounds, uint32_t(s.prep.nmat)), 256, 0, s.stream>>>(out, uint32_t(s.layout.count),
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
        W.span = (uint32_t(p.nz) + 4u) & ~3u;  // nz + 1 rounded up to a multiple of 4
        W.layers = p.paths ? pixels * 2u * W.span : 0u;
        W.count = 4u * pixels + W.layers;
        W.locations = uint32_t(p.nx * p.ny * p.nz * p.angles);
        W.orders = cfg.orders ? W.count : 0u;
        if (cfg.orders) W.count += 4u * (pixels + 2u * W.locations);
        W.vee = p.nmat == 4 ? W.count : 0u;
        if (p.nmat == 4) W.count += pixels;
        W.count = (W.count + 3u) & ~3u;  // every shard's records start 16-byte aligned (vector atomics)
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
        s->held = 0;
        s->held_next = 0;
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
        accumulate(*s, 0, c.rounds, photons_per_column, history);
        s->held = 0;
        s->held_next = 0;
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_run_held(void* handle, const uint32_t controls[8], char* err, size_t errlen) {
    Session* s = static_cast<Session*>(handle);
    if (!s || !controls) { write_error(err, errlen, "Invalid CUDA session or buffers"); return 1; }
    try {
        s->held = 0;
        s->held_next = 0;
        const Controls c = group_controls(*s, controls);
        execute(*s, c);
        finish(*s, c);
        s->held = c.rounds;
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_fold_next(void* handle, double photons_per_column, double* history, char* err, size_t errlen) {
    Session* s = static_cast<Session*>(handle);
    if (!s || !history) { write_error(err, errlen, "Invalid CUDA session or buffers"); return 1; }
    try {
        if (!(photons_per_column > 0.0)) throw std::runtime_error("photons_per_column must be positive");
        if (s->held_next >= s->held) throw std::runtime_error("no held round left to fold");
        accumulate(*s, s->held_next, 1, photons_per_column, history);
        s->held_next += 1;
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
