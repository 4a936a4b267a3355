// Host entry of the tail launch (tail.cu).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include "scene.h"

namespace monki {

struct Controls;
struct Divisors;
struct WaveTally;
template <typename T> struct Pool;

// Runs every photon left in the pool to its end on `stream`: with `pending`, first the
// events queued in work-list buffer b (peeled, not yet scattered: the fused step's last
// iteration), then every other live slot; each launch is a resident wave whose threads take
// entries through the counter *next. Call it only once every photon of the group is claimed.
// max_blocks > 0 caps each launch's grid (a scene with few photons left, sharing the GPU
// with other scenes' tails on other streams).
template <typename T>
cudaError_t launch_tail(const SceneView<T>& v, const Controls& c, const Divisors& dv, const Pool<T>& P, T* banks,
                        const WaveTally& W, const Guide<T>& g, uint32_t b, bool pending, uint32_t* failure,
                        unsigned long long* counters, uint32_t* next, cudaStream_t stream, unsigned max_blocks = 0);

}  // namespace monki
