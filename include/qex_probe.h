/*
 * qex_probe.h -- pipe-throughput probe used as the roofline denominator of
 * the 1D SCF kernel (the machine's measured peaks cover HBM copy bandwidth and
 * bf16 GEMM throughput, not FP64 FMA throughput).  No counterpart in the
 * reference.
 */
#ifndef QEX_PROBE_H_
#define QEX_PROBE_H_

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Measures FP64 and FP32 FMA throughput (TFLOP/s, 2 flops per FMA) on the
 * current device with a grid of 8 CTAs per SM; synchronises the stream.
 * workspace must hold at least qex_probe_workspace_size() bytes. */
size_t qex_probe_workspace_size(void);
int qex_probe_fma_peak(double* fp64_tflops, double* fp32_tflops, void* workspace,
                       size_t workspace_bytes, void* stream);

/* Measures FP64 tensor-core (DMMA, mma.sync) throughput in TFLOP/s for the
 * m8n8k4 and m16n8k16 shapes with the same grid; synchronises the stream.
 * Used to decide whether the FP64 contractions of the 3D path belong on the
 * tensor pipe. */
int qex_probe_dmma_peak(double* m8n8k4_tflops, double* m16n8k16_tflops, void* workspace,
                        size_t workspace_bytes, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* QEX_PROBE_H_ */
