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

#ifdef __cplusplus
}
#endif
#endif /* WAVETORCH_GB300_TESTING_H */
