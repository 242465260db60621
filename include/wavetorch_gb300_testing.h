/*
 * wavetorch_gb300 -- test hooks of the C ABI (not part of the drop-in
 * interface; no counterpart in the reference).
 */
#ifndef WAVETORCH_GB300_TESTING_H
#define WAVETORCH_GB300_TESTING_H

#include "wavetorch_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* wt_seq_fwd for a sequence planned in the band layout, with band `band`
 * (of instance 0's bands) never sending its boundary rows: a host-forced
 * missing arrival.  Its neighbours' bounded waits give up after about 2 s,
 * the launch's abort word stops every band at its next barrier, and
 * wt_seq_device_status then reports WT_ERR_TIMEOUT; the context stays
 * usable.  Nothing faults or hangs.  WT_ERR_UNSUPPORTED when the sequence
 * does not plan in the band layout.                                        */
int wt_test_band_missing_arrival(const wt_scalars* s, const wt_seq_desc* d, const float* b,
                                 const float* c, const float* x, float* out, void* workspace,
                                 size_t workspace_bytes, int32_t band, wt_stream_t stream);

/* wt_seq_fwd for a sequence planned in the cluster layout (at least two
 * CTAs per instance), with CTA `cta` of instance 0's cluster never sending
 * its boundary rows over distributed shared memory: a host-forced missing
 * arrival.  The neighbouring CTAs' bounded waits give up after about 2 s,
 * each CTA leaves its loop at its next abort check, and wt_seq_device_status
 * then reports WT_ERR_TIMEOUT; the context stays usable.  Nothing faults or
 * hangs.  WT_ERR_UNSUPPORTED outside the cluster layout.                   */
int wt_test_cluster_missing_arrival(const wt_scalars* s, const wt_seq_desc* d, const float* b,
                                    const float* c, const float* x, float* out, void* workspace,
                                    size_t workspace_bytes, int32_t cta, wt_stream_t stream);

/* wt_seq_bwd for a sequence whose cluster-layout adjoint runs from the tape,
 * or from checkpoints with the recompute beside the adjoint (after a
 * wt_seq_fwd on the same workspace), with the ring's producer issuing no
 * slice from step `step` down: the CTAs' bounded waits on that slot give up
 * after about 2 s, the copies already in flight are drained, and
 * wt_seq_device_status reports WT_ERR_TIMEOUT; the context stays usable.
 * WT_ERR_UNSUPPORTED when the sequence runs neither way.                    */
int wt_test_tape_missing_slice(const wt_scalars* s, const wt_seq_desc* d, const float* b,
                               const float* c, const float* x, const float* grad_out,
                               float* grad_c, void* workspace, size_t workspace_bytes,
                               int32_t step, wt_stream_t stream);

/* Device peaks that bound the fused sequence kernels (they keep their fields
 * on chip, so HBM does not): measured with two kernels on every SM of the
 * current device, each timed with CUDA events after one warm-up launch.
 *   ffma_per_s       FP32 fused multiply-adds per second (thread operations;
 *                    independent chains, so the loop runs at the issue rate)
 *   warp_inst_per_s  issued warp instructions per second of that loop
 *   smem_bytes_per_s shared-memory load bandwidth (conflict-free 16-byte loads)
 *   sm_mhz           SM clock during the FFMA loop (clock64 / global timer)
 * `scratch` is a device buffer of at least
 * wt_test_device_peaks_scratch_floats() floats (the kernels' outputs).      */
typedef struct wt_device_peaks {
    double ffma_per_s;
    double warp_inst_per_s;
    double smem_bytes_per_s;
    double sm_mhz;
    int32_t sm_count;
} wt_device_peaks;
int wt_test_device_peaks_scratch_floats(size_t* n);
int wt_test_device_peaks(wt_device_peaks* out, float* scratch, size_t scratch_floats,
                         wt_stream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* WAVETORCH_GB300_TESTING_H */
