/*
 * Device-memory probes of libpgb_probes.so, a measurement helper built beside the
 * renderer (not part of its C ABI). Status codes are the renderer's PGB_* codes. No
 * counterpart in the reference.
 */
#ifndef PGB_PROBES_H
#define PGB_PROBES_H

#include <stdint.h>

#include "plenoxels_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* num_reads independent 16 B loads, or num_updates float4 atomic adds of 1, at
 * pseudo-random 16 B slots of a 16-byte-aligned device buffer of table_bytes bytes (every
 * slot inside it). Timed by the caller around the launch, they give the random 32 B
 * sector rate that random cell gathers and gradient scatters run against. sink: one
 * device float, written only if the loaded values sum to -1. */
int pgb_probe_random_reads(const void* table, int64_t table_bytes, int64_t num_reads, uint64_t seed,
                           float* sink, pgb_stream_t stream);
int pgb_probe_random_atomics(void* table, int64_t table_bytes, int64_t num_updates, uint64_t seed,
                             pgb_stream_t stream);

#ifdef __cplusplus
}
#endif

#endif /* PGB_PROBES_H */
