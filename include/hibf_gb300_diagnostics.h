/* hibf_gb300_diagnostics.h -- measurement helpers exported by libhibf_gb300.so beside the product API.
 *
 * Neither replaces a reference interface; they serve the benchmark (bench.py) and profiling.  Nothing in the
 * product calls them, and a seqan::hibf integration needs neither.
 */
#ifndef HIBF_GB300_DIAGNOSTICS_H
#define HIBF_GB300_DIAGNOSTICS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* The device's rate of independent random 8-byte reads over a buffer of footprint_bytes (region_bytes: reads
 * confined to windows of that size, 0 = the whole buffer): the practical ceiling for the query kernels' random row
 * reads, which the copy-bandwidth peak overstates.  Allocates and frees its buffer. */
int hibf_gpu_probe_random_reads(uint64_t footprint_bytes, uint64_t region_bytes, double * reads_per_s);

/* Sets the L2 fetch granularity hint of the calling process's CUDA context (cudaLimitMaxL2FetchGranularity, bytes
 * in [0, 128]); the limit applies to every kernel of the context and ends with it (an experiment knob: random
 * 8-32 byte row reads fetch whole sectors either way). */
int hibf_gpu_set_l2_fetch_granularity(int bytes);

#ifdef __cplusplus
}
#endif

#endif /* HIBF_GB300_DIAGNOSTICS_H */
