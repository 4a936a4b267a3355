// Many scenes in one launch sequence on one GB300: the batched workload's scenes of uneven
// size share one photon pool and run together in each wavefront launch, instead of one
// session (and one stream of small launches) per scene.
//
// The pool is cut into one segment per scene, sized by the scene's photons in the group
// and a multiple of 256 slots; each segment has its own work lists, counts and claim
// counter, so a vacant slot only ever claims its own scene's next photon (the device work
// queue is the scenes' claim counters). A step or peel launch covers every segment:
// thread block b serves 256 list entries of the scene block_scene[b], copies that scene's
// entry (scene view, controls, divisors, pool segment, tally bank) into shared memory,
// stages that scene's extinction band, and runs the same per-slot scattering, walk and
// peel-off functions as the single-scene session. Every scene keeps its own random
// streams (Philox counters keyed by its photons, rounds and seed), so each scene's
// tallies are those of the scene run alone. Scenes are grouped by Stokes size (I or
// I/Q/U), each group on its own stream, the groups' batches interleaved; a batch of
// wavefront iterations is replayed as a CUDA graph built node by node.
//
// The reference batches rounds, not scenes: one dispatch per round group with separate
// random keys and tally banks (python/monki/execution/metal.py:219-242,
// kernels/metal/transport.metal:354-357).
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdio>
#include <memory>
#include <string>
#include <tuple>
#include <utility>
#include <vector>

#include "host_tables.h"
#include "tail.h"
#include "wavefront.cuh"

namespace monki {

// One scene of a multi-scene group as the kernels see it.
template <typename T>
struct SceneEntry {
    SceneView<T> s;
    Controls ctl;
    Divisors dv;
    Pool<T> P;          // the scene's pool segment, work lists and counts
    T* banks;           // rounds x shards x W.count
    WaveTally W;
    unsigned long long* counters;  // the scene's scatters, cell visits, detector visits, tally updates
    uint32_t block0;    // first block (of 256 slots) of the segment in the launches
    uint32_t blocks;    // blocks of the segment
};

constexpr int kMultiBlock = 256;
constexpr int kSceneCounters = 4;  // device counters per scene: scatters, cell visits, detector visits, tally updates
constexpr int kSceneTotals = 6;    // host totals per scene: the four counters, photons, tail launches

// The entry of this block's scene, copied into shared memory by the whole block.
template <typename T>
__device__ __forceinline__ void load_entry(SceneEntry<T>& E, const SceneEntry<T>* __restrict__ scenes,
                                           const uint16_t* __restrict__ block_scene) {
    static_assert(sizeof(SceneEntry<T>) % 4 == 0, "entry copied in 32-bit words");
    const uint32_t* src = reinterpret_cast<const uint32_t*>(scenes + block_scene[blockIdx.x]);
    uint32_t* dst = reinterpret_cast<uint32_t*>(&E);
    for (uint32_t q = threadIdx.x; q < sizeof(SceneEntry<T>) / 4; q += blockDim.x) dst[q] = src[q];
    __syncthreads();
}

// True when this block has no entry of its scene's work lists to serve (lists `first` ..
// `last` of buffer b: 0-2 the event queues, 3 the paused walks, 4 the vacant slots). Such a
// block returns before it copies the entry or stages the band: late in a round group most
// segments are drained and most blocks of a launch are idle.
template <typename T>
__device__ __forceinline__ bool idle_block(const SceneEntry<T>* __restrict__ scenes, const uint16_t* __restrict__ block_scene,
                                           uint32_t b, int first, int last) {
    __shared__ uint32_t idle;
    if (threadIdx.x == 0) {
        const SceneEntry<T>* E = scenes + block_scene[blockIdx.x];
        const uint32_t* c = E->P.counts + kListCounts * b;
        uint32_t total = 0;
        for (int q = first; q <= last; ++q) total += c[q];
        idle = (blockIdx.x - E->block0) * blockDim.x >= total ? 1u : 0u;
    }
    __syncthreads();
    return idle != 0u;
}

// Start of a round group: every segment's slots empty and vacant, no claims yet.
template <typename T>
__global__ void wf_reset_multi(const SceneEntry<T>* __restrict__ scenes, const uint16_t* __restrict__ block_scene) {
    const SceneEntry<T>& E = scenes[block_scene[blockIdx.x]];
    const Pool<T>& P = E.P;
    const uint32_t slot = (blockIdx.x - E.block0) * blockDim.x + threadIdx.x;
    if (slot < P.capacity) {
        P.meta(slot) = make_uint4(kNone, 0u, 0u, 0u);
        P.vacant[0][slot] = slot;
    }
    if (blockIdx.x == E.block0 && threadIdx.x < kCountWords) P.counts[threadIdx.x] = threadIdx.x == 4 ? P.capacity : 0u;
}

template <typename T, int NMAT>
__global__ void __launch_bounds__(kMultiBlock, 4)
wf_step_multi(const SceneEntry<T>* __restrict__ scenes, const uint16_t* __restrict__ block_scene, Guide<T> g,
              uint32_t walk, uint32_t cur, uint32_t* __restrict__ failure) {
    extern __shared__ __align__(16) unsigned char staged[];
    __shared__ __align__(16) SceneEntry<T> E;
    if (idle_block(scenes, block_scene, cur, 0, 4)) return;
    load_entry(E, scenes, block_scene);
    const T* band = stage_band<T>(E.s, staged, failure);
    step_phase<T, NMAT, false, false>(E.s, band, E.ctl, E.dv, E.P, g, walk, cur, failure, E.counters, blockIdx.x - E.block0,
                                      E.blocks);
}

template <typename T, int NMAT>
__global__ void __launch_bounds__(kMultiBlock, sizeof(T) == 4 ? 4 : 3)
wf_peel_multi(const SceneEntry<T>* __restrict__ scenes, const uint16_t* __restrict__ block_scene, uint32_t b,
              uint32_t* __restrict__ failure) {
    extern __shared__ __align__(16) unsigned char staged[];
    __shared__ __align__(16) SceneEntry<T> E;
    if (idle_block(scenes, block_scene, b, 0, 2)) return;
    load_entry(E, scenes, block_scene);
    const T* band = stage_band<T>(E.s, staged, failure);
    peel_phase<T, T, NMAT, false, false>(E.s, band, E.ctl, E.dv, E.P, E.banks, E.W, b, failure, E.counters,
                                         blockIdx.x - E.block0, E.blocks);
}

namespace {

using namespace host;

struct Scene {
    Prepared prep;
    void* tables = nullptr;      // packed scene (T values then int guides)
    SceneView<float> view32{};
    SceneView<double> view64{};
    void* banks = nullptr;       // round_capacity x shards x W.count (T)
    double* out = nullptr;       // round_capacity x tally count (FP64, RawTallies order)
    double* info = nullptr;      // flush info: zunit, 1 / |mu0|, 1 / mu, mu0 / mu
    WaveTally W{};
    uint32_t tally_count = 0;    // stokes elements (nmat * nx * ny * angles)
    int group = 0;
};

struct Group {
    int nmat = 0;
    std::vector<int> members;
    cudaStream_t stream = nullptr;
    void* pool = nullptr;             // records, steps, lists, counts of every segment
    void* entries = nullptr;          // SceneEntry<T>[members]
    uint16_t* block_scene = nullptr;  // scene of each block, up to pool / 256 blocks
    void* host_entries = nullptr;     // pinned staging of the entries
    uint16_t* host_block_scene = nullptr;
    uint32_t* host_counts = nullptr;  // pinned: members x kCountWords
    uint32_t blocks = 0;              // blocks of the current run
    uint32_t band_bytes = 0;          // largest staged band of the group
    bool active = false;
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

struct Multi {
    int device = 0;
    Config cfg;
    uint32_t round_capacity = 1;
    std::vector<Scene> scenes;
    std::vector<Group> groups;
    uint32_t* failure = nullptr;
    unsigned long long* counters = nullptr;    // per scene: kSceneCounters of the current run
    std::vector<uint64_t> scene_totals;        // per scene: its counters, photons and tail launches, summed over runs
    uint32_t* tail_next = nullptr;             // one counter per scene for its tail launch
    std::vector<cudaStream_t> tail_streams;    // the scenes' tails run side by side
    cudaEvent_t t0 = nullptr, t1 = nullptr, t2 = nullptr;
    uint64_t totals[6] = {0, 0, 0, 0, 0, 0};
    float last_kernel_ms = 0.f, last_run_ms = 0.f;
    std::string name;
};

// Pool layout: per slot its record block, then the work-list entries (10 words per slot),
// then the counts of every member scene. The scenes have no layer paths, so each walk's
// step count rides in its record block (Pool::steps null). Every offset comes from here.
size_t lists_offset(size_t slots, size_t record) { return align_up(slots * record, 256); }
size_t counts_offset(size_t slots, size_t record) {
    return lists_offset(slots, record) + align_up(10 * slots * 4, 256);
}
size_t pool_bytes(size_t slots, size_t members, size_t record) {
    return counts_offset(slots, record) + align_up(members * kCountWords * 4, 256);
}

template <typename T>
void upload_scene(Multi& m, Scene& sc, cudaStream_t stream) {
    Packed<T> k = pack<T>(sc.prep, m.cfg.uniform_prefix, m.cfg.rectangles);
    const size_t bytes = k.values.size() * sizeof(T) + k.guides.size() * sizeof(int);
    check(cudaMalloc(&sc.tables, std::max<size_t>(bytes, 16)), "cudaMalloc(scene)");
    check(cudaMemcpyAsync(sc.tables, k.values.data(), k.values.size() * sizeof(T), cudaMemcpyHostToDevice, stream),
          "upload(scene)");
    if (!k.guides.empty())
        check(cudaMemcpyAsync(static_cast<char*>(sc.tables) + k.values.size() * sizeof(T), k.guides.data(),
                              k.guides.size() * sizeof(int), cudaMemcpyHostToDevice, stream), "upload(guides)");
    check(cudaStreamSynchronize(stream), "upload");
    SceneView<T> v = make_view<T>(sc.prep, k, sc.tables);
    if constexpr (sizeof(T) == 4) sc.view32 = v; else sc.view64 = v;
}

void destroy(Multi* m) {
    if (!m) return;
    cudaSetDevice(m->device);
    for (Group& g : m->groups) {
        if (g.stream) cudaStreamSynchronize(g.stream);
        if (g.exec) cudaGraphExecDestroy(g.exec);
        if (g.graph) cudaGraphDestroy(g.graph);
        cudaFree(g.pool); cudaFree(g.entries); cudaFree(g.block_scene);
        if (g.host_entries) cudaFreeHost(g.host_entries);
        if (g.host_block_scene) cudaFreeHost(g.host_block_scene);
        if (g.host_counts) cudaFreeHost(g.host_counts);
        if (g.stream) cudaStreamDestroy(g.stream);
    }
    for (Scene& sc : m->scenes) { cudaFree(sc.tables); cudaFree(sc.banks); cudaFree(sc.out); cudaFree(sc.info); }
    for (cudaStream_t t : m->tail_streams) { cudaStreamSynchronize(t); cudaStreamDestroy(t); }
    cudaFree(m->failure); cudaFree(m->counters); cudaFree(m->tail_next);
    if (m->t0) cudaEventDestroy(m->t0);
    if (m->t1) cudaEventDestroy(m->t1);
    if (m->t2) cudaEventDestroy(m->t2);
    delete m;
}

// The segments of one run: slots in proportion to each scene's photons in the group, at
// least 256 and at most its photons, in multiples of 256; then the entry table.
template <typename T>
void lay_out(Multi& m, Group& g, const std::vector<Controls>& ctl) {
    const size_t slots = m.cfg.pool;
    uint64_t photons = 0;
    for (int id : g.members) photons += ctl[size_t(id)].count;
    const size_t record = kRecordBytes<T>;
    char* base = static_cast<char*>(g.pool);
    unsigned char* records = reinterpret_cast<unsigned char*>(base);
    uint32_t* lists = reinterpret_cast<uint32_t*>(base + lists_offset(slots, record));
    uint32_t* counts = reinterpret_cast<uint32_t*>(base + counts_offset(slots, record));
    SceneEntry<T>* entries = static_cast<SceneEntry<T>*>(g.host_entries);
    uint32_t slot0 = 0, block = 0;
    g.band_bytes = 0;
    for (size_t q = 0; q < g.members.size(); ++q) {
        const int id = g.members[q];
        Scene& sc = m.scenes[size_t(id)];
        const Controls& c = ctl[size_t(id)];
        uint64_t want = photons ? uint64_t(double(slots) * double(c.count) / double(photons)) : 0;
        want = std::min<uint64_t>(want, uint64_t(c.count));
        uint32_t capacity = c.count ? uint32_t(std::max<uint64_t>(256, (want + 255) / 256 * 256)) : 0u;
        if (slot0 + capacity > slots) capacity = uint32_t((slots - slot0) / 256 * 256);
        if (c.count && !capacity) throw std::runtime_error("photon pool too small for the scenes of this group");
        SceneEntry<T>& E = entries[q];
        E = SceneEntry<T>{};
        if constexpr (sizeof(T) == 4) E.s = sc.view32; else E.s = sc.view64;
        g.band_bytes = std::max(g.band_bytes, E.s.band_bytes);
        E.ctl = c;
        E.dv = Divisors{FastDiv::make(c.per_round), FastDiv::make(uint32_t(sc.prep.nx)), FastDiv::make(uint32_t(sc.prep.ny)),
                        FastDiv::make(uint32_t(sc.prep.nx * sc.prep.ny))};
        Pool<T>& P = E.P;
        P.capacity = capacity;
        P.records = records + size_t(slot0) * record;
        P.steps = nullptr;
        for (int b = 0; b < 2; ++b) {
            for (int k = 0; k < 3; ++k) P.queue[b][k] = lists + size_t(5 * b + k) * slots + slot0;
            P.paused[b] = lists + size_t(5 * b + 3) * slots + slot0;
            P.vacant[b] = lists + size_t(5 * b + 4) * slots + slot0;
        }
        P.counts = counts + q * kCountWords;
        E.banks = static_cast<T*>(sc.banks);
        E.W = sc.W;
        E.counters = m.counters + size_t(id) * kSceneCounters;
        E.block0 = block;
        E.blocks = capacity / 256;
        for (uint32_t b = 0; b < E.blocks; ++b) g.host_block_scene[block + b] = uint16_t(q);
        block += E.blocks;
        slot0 += capacity;
    }
    g.blocks = block;
    check(cudaMemcpyAsync(g.entries, g.host_entries, g.members.size() * sizeof(SceneEntry<T>), cudaMemcpyHostToDevice,
                          g.stream), "upload(entries)");
    check(cudaMemcpyAsync(g.block_scene, g.host_block_scene, std::max<uint32_t>(block, 1) * sizeof(uint16_t),
                          cudaMemcpyHostToDevice, g.stream), "upload(blocks)");
}

// Graph (or stream launches) of one batch of check_every wavefront iterations of a group:
// clear the output lists' counts of every segment, step, peel; then read all counts back.
template <typename T, int NMAT>
void batch(Multi& m, Group& g, cudaStream_t stream, cudaGraph_t graph) {
    cudaGraphNode_t last = nullptr;
    auto add = [&](cudaError_t e, cudaGraphNode_t node, const char* what) { check(e, what); last = node; };
    const SceneEntry<T>* entries = static_cast<const SceneEntry<T>*>(g.entries);
    const uint16_t* block_scene = g.block_scene;
    const Guide<T> guide{T(0), T(0), T(INFINITY), nullptr, T(0)};
    uint32_t* const counts =
        reinterpret_cast<uint32_t*>(static_cast<char*>(g.pool) + counts_offset(m.cfg.pool, kRecordBytes<T>));
    const size_t members = g.members.size();
    for (uint32_t it = 0; it < m.cfg.check_every; ++it) {
        uint32_t cur = it & 1u, out = cur ^ 1u;  // kernel arguments: copied when the node or launch is made
        cudaMemsetParams ms{};
        ms.dst = counts + kListCounts * out;
        ms.pitch = kCountWords * sizeof(uint32_t);
        ms.value = 0u;
        ms.elementSize = sizeof(uint32_t);
        ms.width = kListCounts;
        ms.height = members;
        if (graph) {
            cudaGraphNode_t node = nullptr;
            add(cudaGraphAddMemsetNode(&node, graph, last ? &last : nullptr, last ? 1 : 0, &ms), node, "graph memset node");
        } else {
            check(cudaMemset2DAsync(ms.dst, ms.pitch, 0, kListCounts * sizeof(uint32_t), members, stream), "memset(lists)");
        }
        uint32_t walk = m.cfg.walk;
        void* step_args[] = {const_cast<const SceneEntry<T>**>(&entries), const_cast<const uint16_t**>(&block_scene),
                             const_cast<Guide<T>*>(&guide), &walk, &cur, &m.failure};
        void* peel_args[] = {const_cast<const SceneEntry<T>**>(&entries), const_cast<const uint16_t**>(&block_scene), &out,
                             &m.failure};
        const void* fns[2] = {reinterpret_cast<const void*>(&wf_step_multi<T, NMAT>),
                              reinterpret_cast<const void*>(&wf_peel_multi<T, NMAT>)};
        void** args[2] = {step_args, peel_args};
        for (int k = 0; k < 2; ++k) {
            if (graph) {
                cudaKernelNodeParams p{};
                p.func = const_cast<void*>(fns[k]);
                p.gridDim = dim3(g.blocks);
                p.blockDim = dim3(kMultiBlock);
                p.sharedMemBytes = g.band_bytes;
                p.kernelParams = args[k];
                cudaGraphNode_t node = nullptr;
                add(cudaGraphAddKernelNode(&node, graph, last ? &last : nullptr, last ? 1 : 0, &p), node, "graph kernel node");
            } else {
                check(cudaLaunchKernel(fns[k], dim3(g.blocks), dim3(kMultiBlock), args[k], g.band_bytes, stream),
                      "multi-scene launch");
            }
        }
    }
    const size_t bytes = members * kCountWords * sizeof(uint32_t);
    if (graph) {
        cudaGraphNode_t node = nullptr;
        add(cudaGraphAddMemcpyNode1D(&node, graph, last ? &last : nullptr, last ? 1 : 0, g.host_counts, counts, bytes,
                                     cudaMemcpyDeviceToHost), node, "graph copy node");
    } else {
        check(cudaMemcpyAsync(g.host_counts, counts, bytes, cudaMemcpyDeviceToHost, stream), "copy(counts)");
    }
}

template <typename T>
void set_attributes(const Group& g) {
    // Shared memory: the staged band (dynamic) plus the entry and the kernels' own statics.
    const void* step = g.nmat == 1 ? reinterpret_cast<const void*>(&wf_step_multi<T, 1>)
                                   : reinterpret_cast<const void*>(&wf_step_multi<T, 3>);
    const void* peel = g.nmat == 1 ? reinterpret_cast<const void*>(&wf_peel_multi<T, 1>)
                                   : reinterpret_cast<const void*>(&wf_peel_multi<T, 3>);
    for (const void* fn : {step, peel})
        check(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(kBandMaxBytes)), "attribute");
}

template <typename T>
void run(Multi& m, const std::vector<Controls>& ctl) {
    for (Group& g : m.groups) {
        if (g.exec) { cudaGraphExecDestroy(g.exec); g.exec = nullptr; }
        if (g.graph) { cudaGraphDestroy(g.graph); g.graph = nullptr; }
        g.active = false;
        bool any = false;
        for (int id : g.members) any = any || ctl[size_t(id)].count > 0;
        if (!any) continue;
        lay_out<T>(m, g, ctl);
        wf_reset_multi<T><<<g.blocks, kMultiBlock, 0, g.stream>>>(static_cast<const SceneEntry<T>*>(g.entries), g.block_scene);
        check(cudaGetLastError(), "reset launch");
        if (m.cfg.graphs) {
            check(cudaGraphCreate(&g.graph, 0), "graph create");
            if (g.nmat == 1) batch<T, 1>(m, g, g.stream, g.graph); else batch<T, 3>(m, g, g.stream, g.graph);
            check(cudaGraphInstantiate(&g.exec, g.graph, 0), "graph instantiate");
        }
        g.active = true;
    }
    uint64_t it = 0, launches = 0;
    uint64_t limit = 0;
    for (const Controls& c : ctl) limit = std::max<uint64_t>(limit, uint64_t(c.max_steps) + 16);
    for (;;) {
        bool any = false;
        for (Group& g : m.groups) {
            if (!g.active) continue;
            any = true;
            if (g.exec) check(cudaGraphLaunch(g.exec, g.stream), "graph launch");
            else if (g.nmat == 1) batch<T, 1>(m, g, g.stream, nullptr);
            else batch<T, 3>(m, g, g.stream, nullptr);
            launches += 2 * uint64_t(m.cfg.check_every);
        }
        if (!any) break;
        it += m.cfg.check_every;
        for (Group& g : m.groups) {
            if (!g.active) continue;
            check(cudaStreamSynchronize(g.stream), "multi-scene wavefront");
            bool done = true, claimed = true;
            uint64_t live_total = 0;
            for (size_t q = 0; q < g.members.size(); ++q) {
                const uint32_t* h = g.host_counts + q * kCountWords;
                const Controls& c = ctl[size_t(g.members[q])];
                if (!c.count) continue;  // no segment this run: its counts are not in use
                const uint64_t live = uint64_t(h[0]) + h[1] + h[2] + h[3] + h[4];
                done = done && h[kClaimCount] >= c.count && live == 0;
                claimed = claimed && h[kClaimCount] >= c.count;
                live_total += live;
            }
            if (!done && claimed && m.cfg.tail && live_total <= m.cfg.tail) {
                // Few photons left and none to claim: each scene that still has some runs them
                // to their ends in its own tail launch, sized to its photons, side by side on
                // the tail streams (the queued events of the last iteration first).
                const SceneEntry<T>* host = static_cast<const SceneEntry<T>*>(g.host_entries);
                const Guide<T> guide{T(0), T(0), T(INFINITY), nullptr, T(0)};
                size_t used = 0;
                for (size_t q = 0; q < g.members.size(); ++q) {
                    const uint32_t* h = g.host_counts + q * kCountWords;
                    const uint64_t live = uint64_t(h[0]) + h[1] + h[2] + h[3] + h[4];
                    if (!ctl[size_t(g.members[q])].count || !live) continue;
                    const SceneEntry<T>& E = host[q];
                    cudaStream_t t = m.tail_streams[used++ % m.tail_streams.size()];
                    const unsigned blocks = unsigned(std::max<uint64_t>(1, (live + 255) / 256));
                    check(launch_tail<T>(E.s, E.ctl, E.dv, E.P, E.banks, E.W, guide, 0u, true, m.failure, E.counters,
                                         m.tail_next + g.members[q], t, blocks), "tail launch");
                    launches += 2;
                    m.scene_totals[size_t(g.members[q]) * kSceneTotals + 5] += 1;
                }
                for (size_t k = 0; k < std::min(used, m.tail_streams.size()); ++k)
                    check(cudaStreamSynchronize(m.tail_streams[k]), "tail");
                done = true;
            }
            if (done) g.active = false;
        }
        if (it > limit * 4 + 1024 && it > 1000000) throw std::runtime_error("multi-scene wavefront did not drain");
    }
    m.totals[5] += launches;
}

template <typename T>
void flush(Multi& m, const std::vector<Controls>& ctl, cudaStream_t stream) {
    for (Scene& sc : m.scenes) {
        const Controls& c = ctl[size_t(&sc - m.scenes.data())];
        const Prepared& p = sc.prep;
        const uint64_t total = uint64_t(sc.tally_count) * c.rounds;
        const int grid = int(std::max<uint64_t>(1, std::min<uint64_t>((total + 255) / 256, 4096)));
        wf_flush<T><<<grid, 256, 0, stream>>>(static_cast<const T*>(sc.banks), sc.W, p.nmat, p.nx, p.ny, p.nz, p.angles,
                                              sc.info, c.rounds, sc.tally_count, false, sc.out);
        check(cudaGetLastError(), "flush launch");
        check(cudaMemsetAsync(sc.banks, 0, size_t(c.rounds) * sc.W.shards * sc.W.count * sizeof(T), stream),
              "memset(banks)");
    }
}

void write_error(char* err, size_t n, const std::string& msg) {
    if (err && n) std::snprintf(err, n, "%s", msg.c_str());
}

}  // namespace
}  // namespace monki

using namespace monki;

extern "C" {

void* monki_cuda_multi_create(uint32_t device, uint32_t scenes, const double* const* tables, const size_t* table_counts,
                              uint32_t round_capacity, const char* config, char* err, size_t errlen) {
    Multi* m = nullptr;
    try {
        if (!scenes || scenes > 65535 || !tables || !table_counts) throw std::runtime_error("1 to 65535 scenes are needed");
        if (round_capacity < 1 || round_capacity > 4096) throw std::runtime_error("round_capacity must be in [1, 4096]");
        Config cfg = parse_config(config);
        if (!cfg.wavefront || cfg.epsilon > 0.0 || cfg.roulette > 0.0 || cfg.importance || cfg.orders || cfg.split > 0.0)
            throw std::runtime_error("the multi-scene session runs the analog wavefront transport only");
        if (cfg.block != kMultiBlock) throw std::runtime_error("the multi-scene session uses blocks of 256 threads");
        if (cfg.pool % 256) throw std::runtime_error("pool must be a multiple of 256 slots");
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) throw std::runtime_error("No CUDA device is available");
        if (device >= uint32_t(count)) throw std::runtime_error("Requested CUDA device is unavailable");
        m = new Multi();
        m->device = int(device);
        m->cfg = cfg;
        m->round_capacity = round_capacity;
        check(cudaSetDevice(m->device), "cudaSetDevice");
        cudaDeviceProp prop{};
        check(cudaGetDeviceProperties(&prop, m->device), "cudaGetDeviceProperties");
        if (prop.major < 10) throw std::runtime_error("This build targets sm_103a (GB300)");
        m->name = prop.name;
        m->scenes.resize(scenes);
        for (uint32_t q = 0; q < scenes; ++q) {
            Scene& sc = m->scenes[q];
            sc.prep = parse(tables[q], table_counts[q]);
            const Prepared& p = sc.prep;
            if (p.backward || p.paths || (p.nmat != 1 && p.nmat != 3))
                throw std::runtime_error("multi-scene scenes are forward, without layer paths, with nmat 1 or 3");
            const uint32_t pixels = uint32_t(p.nx * p.ny * p.angles);
            sc.W.pixels = pixels;
            sc.W.layers = 0;
            sc.W.count = 4u * pixels;
            sc.W.shards = cfg.shards;
            sc.tally_count = uint32_t(p.nmat) * pixels;
            int group = -1;
            for (size_t g = 0; g < m->groups.size(); ++g)
                if (m->groups[g].nmat == p.nmat) group = int(g);
            if (group < 0) {
                m->groups.emplace_back();
                m->groups.back().nmat = p.nmat;
                group = int(m->groups.size()) - 1;
            }
            sc.group = group;
            m->groups[size_t(group)].members.push_back(int(q));
        }
        const size_t elem = cfg.fp64 ? sizeof(double) : sizeof(float);
        const size_t record = cfg.fp64 ? kRecordBytes<double> : kRecordBytes<float>;
        for (Group& g : m->groups) {
            check(cudaStreamCreateWithFlags(&g.stream, cudaStreamNonBlocking), "cudaStreamCreate");
            check(cudaMalloc(&g.pool, pool_bytes(cfg.pool, g.members.size(), record)), "cudaMalloc(pool)");
            const size_t entry = cfg.fp64 ? sizeof(SceneEntry<double>) : sizeof(SceneEntry<float>);
            check(cudaMalloc(&g.entries, g.members.size() * entry), "cudaMalloc(entries)");
            check(cudaMalloc(&g.block_scene, (cfg.pool / 256) * sizeof(uint16_t)), "cudaMalloc(blocks)");
            check(cudaMallocHost(&g.host_entries, g.members.size() * entry), "cudaMallocHost(entries)");
            check(cudaMallocHost(&g.host_block_scene, (cfg.pool / 256) * sizeof(uint16_t)), "cudaMallocHost(blocks)");
            check(cudaMallocHost(&g.host_counts, g.members.size() * kCountWords * sizeof(uint32_t)), "cudaMallocHost(counts)");
            if (cfg.fp64) set_attributes<double>(g); else set_attributes<float>(g);
        }
        cudaStream_t stream = m->groups.front().stream;
        for (Scene& sc : m->scenes) {
            const Prepared& p = sc.prep;
            if (cfg.fp64) upload_scene<double>(*m, sc, stream); else upload_scene<float>(*m, sc, stream);
            const size_t bank = size_t(round_capacity) * sc.W.shards * sc.W.count * elem;
            check(cudaMalloc(&sc.banks, bank), "cudaMalloc(banks)");
            check(cudaMemsetAsync(sc.banks, 0, bank, stream), "cudaMemset(banks)");
            check(cudaMalloc(&sc.out, size_t(round_capacity) * sc.tally_count * sizeof(double)), "cudaMalloc(out)");
            std::vector<double> info(size_t(p.nz) + 1 + 2 * size_t(p.angles));
            for (int z = 0; z < p.nz; ++z) info[size_t(z)] = p.zunit[size_t(z)];
            const double c0 = std::cos(kDegToRad * p.vartheta0);
            info[size_t(p.nz)] = 1.0 / std::fabs(cfg.fp64 ? c0 : double(float(c0)));
            for (int ia = 0; ia < p.angles; ++ia) {
                const double vc = std::cos(kDegToRad * p.vartheta[size_t(ia)]);
                info[size_t(p.nz) + 1 + ia] = 1.0 / std::fabs(cfg.fp64 ? vc : double(float(vc)));
                info[size_t(p.nz) + 1 + p.angles + ia] = std::fabs(c0) / std::fabs(vc);  // mu0/mu (mc.f90:1456-1474)
            }
            check(cudaMalloc(&sc.info, info.size() * sizeof(double)), "cudaMalloc(flush info)");
            check(cudaMemcpyAsync(sc.info, info.data(), info.size() * sizeof(double), cudaMemcpyHostToDevice, stream),
                  "upload(flush info)");
            check(cudaStreamSynchronize(stream), "upload(flush info)");
        }
        check(cudaMalloc(&m->failure, sizeof(uint32_t)), "cudaMalloc(failure)");
        check(cudaMalloc(&m->counters, m->scenes.size() * kSceneCounters * sizeof(unsigned long long)),
              "cudaMalloc(counters)");
        m->scene_totals.assign(m->scenes.size() * kSceneTotals, 0);
        check(cudaMalloc(&m->tail_next, m->scenes.size() * sizeof(uint32_t)), "cudaMalloc(tail)");
        m->tail_streams.resize(8);
        for (cudaStream_t& t : m->tail_streams) check(cudaStreamCreateWithFlags(&t, cudaStreamNonBlocking), "cudaStreamCreate");
        check(cudaEventCreate(&m->t0), "cudaEventCreate");
        check(cudaEventCreate(&m->t1), "cudaEventCreate");
        check(cudaEventCreate(&m->t2), "cudaEventCreate");
        check(cudaStreamSynchronize(stream), "create");
        return m;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        destroy(m);
        return nullptr;
    }
}

size_t monki_cuda_multi_tally_count(void* handle, uint32_t scene) {
    Multi* m = static_cast<Multi*>(handle);
    return (m && scene < m->scenes.size()) ? m->scenes[scene].tally_count : 0;
}

int monki_cuda_multi_run(void* handle, const uint32_t* controls, double* const* out, char* err, size_t errlen) {
    Multi* m = static_cast<Multi*>(handle);
    if (!m || !controls || !out) { write_error(err, errlen, "Invalid multi-scene session or buffers"); return 1; }
    try {
        std::vector<Controls> ctl(m->scenes.size());
        for (size_t q = 0; q < m->scenes.size(); ++q) {
            const uint32_t* w = controls + 8 * q;
            Controls c{w[0], w[1], w[2], w[3], w[4], w[5], w[6], w[7]};
            if (!c.per_round || !c.rounds || c.rounds > m->round_capacity || !c.max_steps || c.max_steps > kMaxHistorySteps ||
                uint64_t(c.first) + c.count > uint64_t(c.per_round) * c.rounds || !out[q])
                throw std::runtime_error("Invalid CUDA round group for scene " + std::to_string(q));
            ctl[q] = c;
        }
        check(cudaSetDevice(m->device), "cudaSetDevice");
        cudaStream_t first = m->groups.front().stream;
        check(cudaMemsetAsync(m->failure, 0, sizeof(uint32_t), first), "memset(failure)");
        const size_t counter_bytes = m->scenes.size() * kSceneCounters * sizeof(unsigned long long);
        check(cudaMemsetAsync(m->counters, 0, counter_bytes, first), "memset(counters)");
        check(cudaEventRecord(m->t0, first), "event");
        // Every group's stream starts after the clears above.
        for (Group& g : m->groups)
            if (g.stream != first) check(cudaStreamWaitEvent(g.stream, m->t0, 0), "wait");
        if (m->cfg.fp64) run<double>(*m, ctl); else run<float>(*m, ctl);
        for (Group& g : m->groups) check(cudaStreamSynchronize(g.stream), "multi-scene wavefront");
        check(cudaEventRecord(m->t1, first), "event");
        if (m->cfg.fp64) flush<double>(*m, ctl, first); else flush<float>(*m, ctl, first);
        check(cudaEventRecord(m->t2, first), "event");
        uint32_t flag = 0;
        std::vector<unsigned long long> cnt(m->scenes.size() * kSceneCounters, 0ull);
        check(cudaMemcpyAsync(&flag, m->failure, sizeof(flag), cudaMemcpyDeviceToHost, first), "copy(failure)");
        check(cudaMemcpyAsync(cnt.data(), m->counters, counter_bytes, cudaMemcpyDeviceToHost, first), "copy(counters)");
        check(cudaStreamSynchronize(first), "flush");
        if (flag) {
            char msg[128];
            std::snprintf(msg, sizeof msg, "CUDA transport failed (flag %u); round rejected", flag);
            throw std::runtime_error(msg);
        }
        for (size_t q = 0; q < m->scenes.size(); ++q)
            check(cudaMemcpyAsync(out[q], m->scenes[q].out, size_t(m->scenes[q].tally_count) * ctl[q].rounds * sizeof(double),
                                  cudaMemcpyDeviceToHost, first), "copy(tallies)");
        check(cudaStreamSynchronize(first), "copy(tallies)");
        check(cudaEventElapsedTime(&m->last_kernel_ms, m->t0, m->t1), "elapsed");
        check(cudaEventElapsedTime(&m->last_run_ms, m->t0, m->t2), "elapsed");
        for (size_t q = 0; q < m->scenes.size(); ++q) {
            uint64_t* t = m->scene_totals.data() + q * kSceneTotals;
            for (int k = 0; k < kSceneCounters; ++k) {
                t[k] += cnt[q * kSceneCounters + size_t(k)];
                m->totals[k] += cnt[q * kSceneCounters + size_t(k)];
            }
            t[4] += ctl[q].count;
            m->totals[4] += ctl[q].count;
        }
        m->totals[5] += m->scenes.size();  // the flushes
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

int monki_cuda_multi_counters(void* handle, uint64_t out[6]) {
    if (!handle || !out) return 1;
    Multi* m = static_cast<Multi*>(handle);
    for (int q = 0; q < 6; ++q) out[q] = m->totals[q];
    return 0;
}

int monki_cuda_multi_scene_counters(void* handle, uint32_t scene, uint64_t out[6]) {
    Multi* m = static_cast<Multi*>(handle);
    if (!m || !out || scene >= m->scenes.size()) return 1;
    for (int k = 0; k < kSceneTotals; ++k) out[k] = m->scene_totals[size_t(scene) * kSceneTotals + size_t(k)];
    return 0;
}

int monki_cuda_multi_last_timing(void* handle, float out[2]) {
    if (!handle || !out) return 1;
    Multi* m = static_cast<Multi*>(handle);
    out[0] = m->last_kernel_ms;
    out[1] = m->last_run_ms;
    return 0;
}

void monki_cuda_multi_close(void* handle) { destroy(static_cast<Multi*>(handle)); }

}  // extern "C"
