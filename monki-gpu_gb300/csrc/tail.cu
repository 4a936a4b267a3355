// Launch of the tail kernel (wf_tail, wavefront.cuh): the end of a round group, once every
// photon is claimed and few remain, in one launch instead of three launches per wavefront
// iteration. Kept in its own translation unit so its many instantiations (scalar, Stokes
// size, layer paths, transport direction) compile in parallel with the rest of the library.
#include <cuda_runtime.h>

#include <algorithm>

#include "tail.h"
#include "wavefront.cuh"

namespace monki {

namespace {

template <typename T, int NMAT, bool PATHS, bool BACKWARD>
cudaError_t launch(const SceneView<T>& v, const Controls& c, const Divisors& dv, const Pool<T>& P, T* banks,
                   const WaveTally& W, const Guide<T>& g, uint32_t b, bool pending, uint32_t* failure,
                   unsigned long long* counters, uint32_t* next, cudaStream_t stream, unsigned max_blocks) {
    const void* fn = reinterpret_cast<const void*>(&wf_tail<T, NMAT, PATHS, BACKWARD>);
    int device = 0, sms = 0, per_sm = 0;
    cudaError_t e = cudaGetDevice(&device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device);
    if (e == cudaSuccess && v.band_bytes)
        e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, int(v.band_bytes));
    if (e == cudaSuccess) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 256, v.band_bytes);
    if (e != cudaSuccess) return e;
    // One resident wave per launch: the threads take entries until none is left. With
    // `pending`, the events queued in buffer b first (they still need their scattering).
    for (const bool first : {true, false}) {
        if (first && !pending) continue;
        e = cudaMemsetAsync(next, 0, sizeof(uint32_t), stream);
        if (e != cudaSuccess) return e;
        unsigned grid = unsigned(std::max(per_sm, 1) * sms);
        if (max_blocks) grid = std::min(grid, max_blocks);
        wf_tail<T, NMAT, PATHS, BACKWARD><<<grid, 256, v.band_bytes, stream>>>(
            v, c, dv, P, banks, W, g, b, first, failure, counters, next);
        e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

}  // namespace

template <typename T>
cudaError_t launch_tail(const SceneView<T>& v, const Controls& c, const Divisors& dv, const Pool<T>& P, T* banks,
                        const WaveTally& W, const Guide<T>& g, uint32_t b, bool pending, uint32_t* failure,
                        unsigned long long* counters, uint32_t* next, cudaStream_t stream, unsigned max_blocks) {
    const bool paths = v.paths != 0, backward = v.backward != 0;
    if (v.nmat == 1 && paths == false && backward == false)
        return launch<T, 1, false, false>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 1 && paths == true && backward == false)
        return launch<T, 1, true, false>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 3 && paths == false && backward == false)
        return launch<T, 3, false, false>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 3 && paths == true && backward == false)
        return launch<T, 3, true, false>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 4 && paths == false && backward == false)
        return launch<T, 4, false, false>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 4 && paths == true && backward == false)
        return launch<T, 4, true, false>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 1 && paths == false && backward == true)
        return launch<T, 1, false, true>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 1 && paths == true && backward == true)
        return launch<T, 1, true, true>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 3 && paths == false && backward == true)
        return launch<T, 3, false, true>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 3 && paths == true && backward == true)
        return launch<T, 3, true, true>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 4 && paths == false && backward == true)
        return launch<T, 4, false, true>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    if (v.nmat == 4 && paths == true && backward == true)
        return launch<T, 4, true, true>(v, c, dv, P, banks, W, g, b, pending, failure, counters, next, stream, max_blocks);
    return cudaErrorInvalidValue;
}

template cudaError_t launch_tail<float>(const SceneView<float>&, const Controls&, const Divisors&, const Pool<float>&,
                                        float*, const WaveTally&, const Guide<float>&, uint32_t, bool, uint32_t*,
                                        unsigned long long*, uint32_t*, cudaStream_t, unsigned);
template cudaError_t launch_tail<double>(const SceneView<double>&, const Controls&, const Divisors&,
                                         const Pool<double>&, double*, const WaveTally&, const Guide<double>&, uint32_t,
                                         bool, uint32_t*, unsigned long long*, uint32_t*, cudaStream_t, unsigned);

}  // namespace monki
