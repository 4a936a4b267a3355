// Device probes of the transport helpers, exported through the C ABI so the parity tests
// can run the production device functions in isolation: the same role as the probe-kernel
// pattern of the reference's device tests (tests/integration/test_metal.py:23-59, 62-103).
#include <cuda_runtime.h>
#include <cstdio>
#include <stdexcept>
#include <string>

#include "physics.cuh"

namespace monki {
namespace {

__global__ void philox_probe(const uint4* ctr, const uint2* key, uint4* out, uint32_t n) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) out[t] = philox4x32_10(ctr[t], key[t]);
}

__global__ void uniform_probe(uint32_t photon, uint32_t round, uint32_t seed, uint32_t n, float* out) {
    if (blockIdx.x || threadIdx.x) return;
    PhotonStream s;
    s.reset(photon, round, seed);
    for (uint32_t q = 0; q < n; ++q) out[q] = s.next();
}

// Rayleigh phase matrix, meridian rotations and the forward product L2 F L1 S for each
// geometry (uo, u1, phio, phi1); the scattering cosine follows from the geometry.
template <typename T>
__global__ void scatter_probe(T depol, const double* geom, const double* stokes, uint32_t n, double* out) {
    uint32_t t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= n) return;
    T uo = T(geom[4 * t]), u1 = T(geom[4 * t + 1]), po = T(geom[4 * t + 2]), p1 = T(geom[4 * t + 3]);
    T cs = uo * u1 + sqrt(T(1) - uo * uo) * sqrt(T(1) - u1 * u1) * cos(po - p1);
    Phase<T> f = rayleigh<T>(cs, depol, 3);
    Rot<T> r = rotation<T>(cs, uo, u1, po, p1);
    T s[3] = {T(stokes[0]), T(stokes[1]), T(stokes[2])}, o[3];
    scatter_stokes<T>(f, r, 3, s, o);
    for (int m = 0; m < 3; ++m) out[3 * t + m] = double(o[m]);
}

void check(cudaError_t e, const char* what) {
    if (e != cudaSuccess) throw std::runtime_error(std::string(what) + ": " + cudaGetErrorString(e));
}

void write_error(char* err, size_t n, const std::string& msg) {
    if (err && n) std::snprintf(err, n, "%s", msg.c_str());
}

template <typename F>
int guarded(uint32_t device, char* err, size_t errlen, F body) {
    try {
        int count = 0;
        if (cudaGetDeviceCount(&count) != cudaSuccess || device >= uint32_t(count))
            throw std::runtime_error("Requested CUDA device is unavailable");
        check(cudaSetDevice(int(device)), "cudaSetDevice");
        body();
        check(cudaDeviceSynchronize(), "probe");
        return 0;
    } catch (const std::exception& e) {
        write_error(err, errlen, e.what());
        return 1;
    }
}

}  // namespace
}  // namespace monki

using namespace monki;

extern "C" {

int monki_cuda_probe_philox(uint32_t device, const uint32_t* counters, const uint32_t* keys, uint32_t n,
                            uint32_t* out, char* err, size_t errlen) {
    return guarded(device, err, errlen, [&] {
        if (!n) return;
        uint4 *dc = nullptr, *dout = nullptr;
        uint2* dk = nullptr;
        check(cudaMalloc(&dc, n * sizeof(uint4)), "cudaMalloc");
        check(cudaMalloc(&dk, n * sizeof(uint2)), "cudaMalloc");
        check(cudaMalloc(&dout, n * sizeof(uint4)), "cudaMalloc");
        check(cudaMemcpy(dc, counters, n * sizeof(uint4), cudaMemcpyHostToDevice), "copy");
        check(cudaMemcpy(dk, keys, n * sizeof(uint2), cudaMemcpyHostToDevice), "copy");
        philox_probe<<<(n + 127) / 128, 128>>>(dc, dk, dout, n);
        check(cudaGetLastError(), "launch");
        check(cudaMemcpy(out, dout, n * sizeof(uint4), cudaMemcpyDeviceToHost), "copy");
        cudaFree(dc); cudaFree(dk); cudaFree(dout);
    });
}

int monki_cuda_probe_uniforms(uint32_t device, uint32_t photon, uint32_t round, uint32_t seed, uint32_t n,
                              float* out, char* err, size_t errlen) {
    return guarded(device, err, errlen, [&] {
        if (!n) return;
        float* d = nullptr;
        check(cudaMalloc(&d, n * sizeof(float)), "cudaMalloc");
        uniform_probe<<<1, 32>>>(photon, round, seed, n, d);
        check(cudaGetLastError(), "launch");
        check(cudaMemcpy(out, d, n * sizeof(float), cudaMemcpyDeviceToHost), "copy");
        cudaFree(d);
    });
}

int monki_cuda_probe_scatter_stokes(uint32_t device, int fp64, double depol, const double* geometry,
                                    const double* stokes, uint32_t n, double* out, char* err, size_t errlen) {
    return guarded(device, err, errlen, [&] {
        if (!n) return;
        double *dg = nullptr, *ds = nullptr, *dout = nullptr;
        check(cudaMalloc(&dg, n * 4 * sizeof(double)), "cudaMalloc");
        check(cudaMalloc(&ds, 3 * sizeof(double)), "cudaMalloc");
        check(cudaMalloc(&dout, n * 3 * sizeof(double)), "cudaMalloc");
        check(cudaMemcpy(dg, geometry, n * 4 * sizeof(double), cudaMemcpyHostToDevice), "copy");
        check(cudaMemcpy(ds, stokes, 3 * sizeof(double), cudaMemcpyHostToDevice), "copy");
        if (fp64) scatter_probe<double><<<(n + 127) / 128, 128>>>(depol, dg, ds, n, dout);
        else scatter_probe<float><<<(n + 127) / 128, 128>>>(float(depol), dg, ds, n, dout);
        check(cudaGetLastError(), "launch");
        check(cudaMemcpy(out, dout, n * 3 * sizeof(double), cudaMemcpyDeviceToHost), "copy");
        cudaFree(dg); cudaFree(ds); cudaFree(dout);
    });
}

}  // extern "C"
