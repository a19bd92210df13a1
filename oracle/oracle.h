/*
 * oracle.h — CPU restatement of Butterfly's SCALAR execution strategy.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and
 * bench.py (its CPU-baseline leg and its reference arm) may load this
 * library, and only as the checker / the timed CPU baseline.  The engine
 * (libbfgpu) never calls it.
 *
 * Parity pinning: the reference is Mojo (mojo 0.25.7, osx-arm64 only) and
 * cannot be built or run here, and it ships no golden vectors for this path.
 * The restatement is pinned against the known-answer checks its own tests
 * hold: gate QFT/IQFT against the classical FFT (tests/test_qft_classical.mojo),
 * bit-reversal involution and full == partial (tests/test_bit_reverse.mojo),
 * U * U^-1 |0> = |0> (tests/test_circuit_inverse.mojo), and analytic states
 * (H^n|0>, value encoding of an integer), against committed fixtures made by
 * an independent numpy FFT (tests/golden/make_golden.py).
 */
#ifndef BF_ORACLE_H
#define BF_ORACLE_H

#include <stddef.h>
#include <stdint.h>

#include "../include/bfgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* strategies restated here (values of ExecutionStrategy, context.mojo:33-40) */
enum {
  OR_SCALAR = 0,         /* sequential scalar kernels: the oracle         */
  OR_SIMD_PARALLEL = 3   /* chunked multi-threaded port: the CPU baseline */
};

/* Runs ops on the SoA state (re, im) of 2^n amplitudes in place.
 * strategy: OR_SCALAR or OR_SIMD_PARALLEL; threads: worker threads for
 * OR_SIMD_PARALLEL (0 = all online cores); chunks: work items per gate
 * (ExecContext.quantum_simd_parallel_chunks; 0 = threads).
 * specialized: BF_SPEC_* mask.  Returns 0 or a negative BF_E* code with the
 * message in err. */
int or_execute(int32_t n, double* re, double* im, const bf_op* ops,
               int64_t nops, int32_t strategy, int32_t threads, int32_t chunks,
               uint32_t specialized, int32_t validate, char* err,
               size_t errlen);

/* Classical QFT / IQFT over targets (butterfly/algos/qft_classical.mojo:
 * 131-222): the FFT the reference's gate QFT is tested against. */
int or_qft_classical(int32_t n, double* re, double* im, const int32_t* targets,
                     int32_t ntargets, int32_t inverse, int32_t swap,
                     char* err, size_t errlen);

/* Full bit reversal of the index (state.mojo:131-204) as an index map:
 * out_index[i] = rev_n(i).  Used to check permutations bit-exactly. */
void or_bit_reverse_indices(int32_t n, uint64_t* out_index);

/* apply_measure (state.mojo:447-553): values[k] -1 = free, 0/1 = fixed. */
int or_measure(int32_t n, double* re, double* im, const int32_t* targets,
               const int8_t* values, int32_t ntargets, int64_t seed,
               uint64_t* outcome, double* prob, char* err, size_t errlen);

/* The k most probable basis states (descending probability, ties by index). */
void or_topk(int32_t n, const double* re, const double* im, int32_t k,
             uint64_t* idx, double* prob);

/* sum |amp|^2 in FP64. */
double or_norm2(int32_t n, const double* re, const double* im);

/* Online host cores the parallel port would use. */
int32_t or_num_cores(void);

/* The reference's circuit fusion rewrites (butterfly/core/
 * transformations_fusion.mojo:879-908) over op records: mode 0
 * fuse_circuit (adjacent-qubit pairs into 4x4 unitaries, then same-target
 * runs), mode 1 fuse_circuit_specialized_pairs (special pairs into fused
 * pair records, then same-target runs).  Writes the rewritten records to
 * out (at most out_cap) and the matrices of the unitaries they produce to
 * mats (interleaved doubles, at most mats_cap; the records' data point
 * there); *nout = records produced.  A second restatement beside the host
 * mirror's, to check it. */
int or_fuse(int32_t mode, const bf_op* in, int64_t nin, bf_op* out,
            int64_t out_cap, double* mats, int64_t mats_cap, int64_t* nout,
            char* err, size_t errlen);

#ifdef __cplusplus
}
#endif

#endif
