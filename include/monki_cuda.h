/* C ABI of libmonki_cuda.so: MONKI photon transport on one GB300 (sm_103a).
 *
 * Each entry point replaces one entry point of the reference's Metal host bridge
 * (kernels/metal/bridge.m, bound from python/monki/execution/metal.py:125-155); the
 * reference has no CUDA path. Plain pointers and sizes only. Every call that can fail
 * returns nonzero (or NULL) and writes a message into err[0..errlen).
 *
 * Transport tables: the float64 stream of kernels/cpu/worker.f90:1102-1120 (version 1)
 * or version 2, which adds one view azimuth per view after the view zeniths.
 *
 * Controls (eight uint32 words, as kernels/metal/README.md:52-55): photon count, first
 * flattened photon of the round group, first statistical round, seed, step limit per
 * history and per detector ray, profiling flag, photons per round, rounds in the group.
 *
 * Output of a run: rounds x tally_count float64 values; each round holds, in Fortran
 * order, stokes(nmat,nx,ny,angles) with the mu0/mu factor applied, then (when the
 * tables request path diagnostics) paths(nx,ny,nz,angles) and weights(nx,ny,angles) -
 * the RawTallies layout of python/monki/execution/tallies.py:21-32.
 *
 * Failure flags in error messages: 1 nonfinite contribution, 2 detector step limit,
 * 4 sampling limit, 8 invalid Stokes vector, 16 history step limit
 * (kernels/metal/README.md:57-59). A failed run rejects the whole round group.
 */
#ifndef MONKI_CUDA_H
#define MONKI_CUDA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces monki_metal_abi_version (kernels/metal/bridge.m:26). Returns 1. */
int monki_cuda_abi_version(void);

/* Replaces monki_metal_create (kernels/metal/bridge.m:30-84). Validates and packs the
 * table stream, uploads it, allocates tally banks for round_capacity rounds. config is
 * "key=value" items separated by ',' or ';': precision=fp32|fp64, shards=1..64,
 * block=32..256, blocks_per_sm=0..64, uniform_prefix=0|1. Returns NULL on failure. */
void *monki_cuda_create(uint32_t device, const double *tables, size_t table_count,
                        uint32_t round_capacity, const char *config, char *err, size_t errlen);

/* Replaces monki_metal_run (kernels/metal/bridge.m:88-133). Runs one round group and
 * copies its FP64 tallies to out (rounds x tally_count). Nonzero on failure. controls:
 * {count, first, first_round, seed, max_steps (1..10,000,000), profile, per_round, rounds}. */
int monki_cuda_run(void *session, const uint32_t controls[8], double *out, char *err,
                   size_t errlen);

/* Replaces monki_metal_gpu_seconds (kernels/metal/bridge.m:135): summed transport time
 * of runs whose profiling flag was set. */
double monki_cuda_gpu_seconds(void *session);

/* Device time of the last run in milliseconds from CUDA events on the session stream:
 * out[0] the transport kernel, out[1] transport plus the FP64 flush. No reference
 * counterpart. */
int monki_cuda_last_timing(void *session, float out[2]);

/* Session totals: scatters, free-path walk steps, detector cell visits, tally updates,
 * photons, kernel launches. No reference counterpart (the scatter count is mc.f90's nscat). */
int monki_cuda_counters(void *session, uint64_t out[6]);

/* Wavefront stage timing of the last run with the profiling flag set, from CUDA events
 * around each launch: summed milliseconds and launch counts of (0) the walks — the fused
 * step kernel, which also scatters the previous iteration's events, or the transit kernel
 * of scenes with layer paths —, (1) the peel-off and (2) the separate scattering kernel of
 * scenes with layer paths (0 when fused). No reference counterpart. */
int monki_cuda_stage_timing(void *session, double ms[3], uint64_t launches[3]);

/* Number of float64 values per round in a run's output; no reference counterpart. */
size_t monki_cuda_tally_count(void *session);

/* Replaces monki_metal_device_name (kernels/metal/bridge.m:140). */
const char *monki_cuda_device_name(void *session);

/* Replaces monki_metal_close (kernels/metal/bridge.m:145-150). Safe on NULL. */
void monki_cuda_close(void *session);

/* Device round statistics (no reference counterpart: the reference driver sums rounds on
 * the host, python/monki/simulation.py:86-103). Runs one round group like monki_cuda_run
 * but keeps its tallies on the device: each round is folded, in round order and in FP64
 * with correctly rounded operations, into the session's statistics (Stokes total, sum and
 * sum of squares of tally / photons_per_column; path and weight sums and the Welford
 * moments of the AMF stopping rule, python/monki/convergence.py:37-99). history receives
 * rounds x nmat values: each round's sum over pixels of its normalized Stokes tallies.
 * A failed group leaves the statistics unchanged. */
int monki_cuda_run_accumulate(void *session, const uint32_t controls[8], double photons_per_column, double *history,
                              char *err, size_t errlen);
/* A round group run ahead of its stopping checks: like monki_cuda_run_accumulate, but the
 * group's flushed rounds are held on the device unfolded; monki_cuda_fold_next then folds
 * them one at a time, in round order, writing that round's nmat history values. Rounds
 * left unfolded when the caller stops are discarded by the next run. Replaces the
 * reference driver's round-by-round dispatch after its minimum rounds
 * (python/monki/simulation.py:86-103) with the same rounds, folds and checks. */
int monki_cuda_run_held(void *session, const uint32_t controls[8], char *err, size_t errlen);
int monki_cuda_fold_next(void *session, double photons_per_column, double *history, char *err, size_t errlen);

/* Length of the statistics vector: total, sum, squares (nmat nx ny angles each); with path
 * diagnostics the path sum, mean, M2 and covariance (nx ny nz angles each) and the weight
 * sum, mean and M2 (nx ny angles each); Fortran order within each block. */
size_t monki_cuda_statistics_count(void *session);

/* Copy the statistics out (count values) with the number of rounds folded in. */
int monki_cuda_statistics(void *session, double *out, size_t count, uint64_t *rounds, char *err, size_t errlen);

/* Clear the statistics; returns nonzero for a NULL session. */
int monki_cuda_reset_statistics(void *session);

/* Guided transport (no reference counterpart: the reference's transport is analog only).
 * Created with config items epsilon=E (detector-directed sampling probability at particle
 * scatters, [0, 1)), roulette=W (Russian-roulette weight, [0, 1], 0 = off) and cap=C (the
 * detector branch only for photons lighter than C, 0 = always); the estimator keeps the
 * analog expectation exactly. This call gives the roulette weight a per-cell scale:
 * scale holds nx * ny * nz non-negative values in Fortran cell order (i fastest, the
 * vacuum layer included); NULL removes the map. Applies to later runs. Returns nonzero
 * with a message in err on failure. */
int monki_cuda_set_roulette_scale(void *session, const double *scale, size_t cells, char *err, size_t errlen);

/* Importance tally of a session created with importance=1 (no reference counterpart):
 * writes 2 * nx * ny * nz values, per cell the summed Stokes-I peel-off contribution, per
 * unit weight at the event, of every event there and of the next seven events of its
 * history, then the event count; reset != 0 clears the tally. */
int monki_cuda_importance(void *session, double *out, size_t count, int reset, char *err, size_t errlen);

/* Weights of the importance tally's contributions per output pixel (nx * ny * angles,
 * Fortran order, non-negative; NULL restores 1): a contribution to pixel p counts
 * weights[p] times, so the tally measures importance for a weighted objective (for
 * example the pixels whose relative error limits a precision target). */
int monki_cuda_set_importance_weights(void *session, const double *weights, size_t pixels, char *err, size_t errlen);

/* Host-only check of the table packer (no GPU needed): validates the stream and returns
 * the first layer of the horizontally uniform top and the optical depth above each
 * layer, at fp32 or fp64 transport precision. The counterpart of the uniform-top prefix
 * of python/monki/execution/metal_tables.py:93-107. */
int monki_cuda_inspect(const double *tables, size_t table_count, int fp64, int32_t *uniform_top,
                       double *tau_above, size_t tau_capacity, char *err, size_t errlen);

/* Host-only check of the equal-extinction rectangles (no GPU needed; no counterpart in
 * the reference, whose walks step face by face). Writes, for every cell below the
 * uniform top (i + nx * (j + ny * k)), the word the cell walks read: bytes 0-3 are the
 * cells of its rectangle before it along -x, after it along +x, before it along -y and
 * after it along +y (each at most 255). *written receives the cell count (0 when the
 * scene has no horizontally varying layer). */
int monki_cuda_inspect_rectangles(const double *tables, size_t table_count, int fp64, uint32_t *extent,
                                  size_t capacity, size_t *written, char *err, size_t errlen);

/* Transport without device allocation; no counterpart in the reference. For callers
 * that cannot call cudaMalloc (an application that owns all device memory through its
 * own arena, a real-time loop that must not allocate while running, a plugin host that
 * owns the GPU memory budget): runs one round group of the photon-history kernel like
 * monki_cuda_run, but keeps every device scratch buffer (packed scene, FP32 tally bank,
 * FP64 output staging, flags) in one fixed 16 MiB array inside this library, which each
 * GPU that loads the library holds until the process exits. Inputs and outputs are the
 * caller's host arrays, as for create + run. Scenes whose scratch exceeds 16 MiB are
 * rejected with an error. All calls share the array: calls that overlap on the GPU race,
 * and each call clears what must start at zero. The first call on a device looks up the
 * array's device address and keeps it for the process's lifetime; make it before any
 * stream capture, and do not reset the device between calls. A call that returns nonzero
 * leaves `out` untouched. */
int monki_cuda_run_static(uint32_t device, const double *tables, size_t table_count,
                          const uint32_t controls[8], double *out, char *err, size_t errlen);

/* Many scenes in one launch sequence (no counterpart in the reference, which batches the
 * rounds of one scene: python/monki/execution/metal.py:219-242). Each scene is a prepared
 * table stream as for monki_cuda_create (forward, no layer paths, nmat 1 or 3); one photon
 * pool is shared by every scene, each wavefront launch covers all of them, and each scene
 * keeps its own random streams and tallies. Config keys as for monki_cuda_create (precision,
 * pool, walk, check_every, graphs, shards, rectangles, uniform_prefix); the analog method
 * only. Returns NULL on failure with the message in err. */
void *monki_cuda_multi_create(uint32_t device, uint32_t scenes, const double *const *tables,
                              const size_t *table_counts, uint32_t round_capacity, const char *config,
                              char *err, size_t errlen);
/* Tally values per round of one scene (nmat * nx * ny * angles). */
size_t monki_cuda_multi_tally_count(void *handle, uint32_t scene);
/* One round group per scene: controls holds eight words per scene (as monki_cuda_run's),
 * out[scene] receives rounds x tally count FP64 values in RawTallies order. A scene with a
 * photon count of 0 sits this run out. Nonzero on failure, with the message in err. */
int monki_cuda_multi_run(void *handle, const uint32_t *controls, double *const *out, char *err, size_t errlen);
/* scatters, free-path cell visits, detector cell visits, tally updates, photons, launches. */
int monki_cuda_multi_counters(void *handle, uint64_t out[6]);
/* One scene's totals over the session's runs: scatters, free-path cell visits, detector cell
 * visits, tally updates, photons, tail launches. Nonzero for an unknown scene. */
int monki_cuda_multi_scene_counters(void *handle, uint32_t scene, uint64_t out[6]);
/* Milliseconds of the last run: transport, and transport plus the FP64 flush. */
int monki_cuda_multi_last_timing(void *handle, float out[2]);
void monki_cuda_multi_close(void *handle);

/* Device probes of the production helpers, the counterpart of the reference's probe
 * kernels (tests/integration/test_metal.py:23-103). */
int monki_cuda_probe_philox(uint32_t device, const uint32_t *counters, const uint32_t *keys,
                            uint32_t n, uint32_t *out, char *err, size_t errlen);
int monki_cuda_probe_uniforms(uint32_t device, uint32_t photon, uint32_t round, uint32_t seed,
                              uint32_t n, float *out, char *err, size_t errlen);
int monki_cuda_probe_scatter_stokes(uint32_t device, int fp64, double depol,
                                    const double *geometry, const double *stokes, uint32_t n,
                                    double *out, char *err, size_t errlen);

#ifdef __cplusplus
}
#endif

#endif /* MONKI_CUDA_H */
