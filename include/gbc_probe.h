/*
 * gbc_probe.h -- measurement only, not part of the verify path: the
 * shared-memory atomic roof the bench reports the sieve stages against.
 * Built as its own library (libgbc_probe.so); the product library libgbc.so
 * does not contain it. No counterpart in the reference.
 */
#ifndef GBC_PROBE_H
#define GBC_PROBE_H

#ifdef __cplusplus
extern "C" {
#endif

/* Conflict-free 32-bit atomicAnd throughput of the device (one CTA of 1024
 * threads per SM, the tile sieve's shape, every warp instruction on 32
 * banks): atomics per second over an event-timed launch and atomics per SM
 * clock; either pointer may be NULL. The caller's current device is the
 * same on return. Returns 0, or -2 (GBC_E_CUDA of gbc.h) when a CUDA call
 * failed or there is no device. */
int gbc_smem_atomic_peak(int device, double *atomics_per_s, double *per_clock_per_sm);

#ifdef __cplusplus
}
#endif

#endif /* GBC_PROBE_H */
