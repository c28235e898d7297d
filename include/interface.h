/*
 * interface.h -- drop-in C API of the GB300 domain propagator.
 *
 * Every symbol of the reference library's public header (include/interface.h
 * of Sofranac-Boro/gpu-domain-propagator) is exported by libgdp_gb300.so with
 * the same name, argument list and argument meaning, so a caller built against
 * the reference (ctypes driver fileReader/GPUDomPropInterface.py, or a MIP
 * solver) links against this library unchanged.
 *
 * Argument contract (reference src/interface.cu, src/propagators/GPU_propagator.cuh):
 *   - all pointers are HOST memory; CSR is 0-based with csr_row_ptrs[n_cons] == nnz;
 *   - lbs / ubs are in/out and receive the propagated bounds;
 *   - vartypes holds GDP_VARTYPE values; anything != GDP_CONTINUOUS is integral;
 *   - n_cons == 0 || n_vars == 0 || nnz == 0 returns GDP_OKAY, bounds untouched.
 * Errors: invalid input, CUDA errors and allocation failures return GDP_ERROR
 * (the reference called exit() on CUDA errors); gdp_last_error() in gdp_ext.h
 * gives the message. Round count and infeasibility are available through the
 * extended API (gdp_ext.h), since these signatures have no room for them.
 *
 * Implemented: the FP64 GPU entry points. FP32 entry points and the CPU
 * algorithms (sequential / OpenMP / measure variants) return
 * GDP_NOTIMPLEMENTED: this library is the GPU FP64 hot path only, with no CPU
 * fallback.
 */
#ifndef GDP_GB300_INTERFACE_H
#define GDP_GB300_INTERFACE_H

#include "gdp_types.h"

#ifdef __cplusplus
#define GDP_DEFAULT_SYNC = 0
extern "C" {
#else
#define GDP_DEFAULT_SYNC
#endif

/* Replaces reference include/interface.h:10-22 (propagateConstraintsGPUReductionDouble).
 * The reference's reduction algorithm is a Jacobi variant without infinity
 * counts; here it runs the same deterministic Jacobi round kernel as the
 * atomic entry point (CPU_LOOP driver). */
GDP_RETCODE propagateConstraintsGPUReductionDouble(
        const int n_cons, const int n_vars, const int nnz,
        const int *csr_col_indices, const int *csr_row_ptrs, const double *csr_vals,
        const double *lhss, const double *rhss,
        double *lbs, double *ubs, const int *vartypes);

/* Replaces reference include/interface.h:32-44. Returns GDP_NOTIMPLEMENTED (FP64 only). */
GDP_RETCODE propagateConstraintsGPUReductionFloat(
        const int n_cons, const int n_vars, const int nnz,
        const int *csr_col_indices, const int *csr_row_ptrs, const float *csr_vals,
        const float *lhss, const float *rhss,
        float *lbs, float *ubs, const int *vartypes);

/* Replaces reference include/interface.h:54-67 (propagateConstraintsGPUAtomicDouble):
 * the primary drop-in. sync_type selects the round-loop driver (GDP_SYNCTYPE);
 * an unknown value returns GDP_ERROR, as the reference's
 * std::runtime_error("Unknown sync type") did (GPU_propagator.cuh:256-259). */
GDP_RETCODE propagateConstraintsGPUAtomicDouble(
        const int n_cons, const int n_vars, const int nnz,
        const int *csr_col_indices, const int *csr_row_ptrs, const double *csr_vals,
        const double *lhss, const double *rhss,
        double *lbs, double *ubs, const int *vartypes,
        const int sync_type GDP_DEFAULT_SYNC);

/* Replaces reference include/interface.h:77-90. Returns GDP_NOTIMPLEMENTED (FP64 only). */
GDP_RETCODE propagateConstraintsGPUAtomicFloat(
        const int n_cons, const int n_vars, const int nnz,
        const int *csr_col_indices, const int *csr_row_ptrs, const float *csr_vals,
        const float *lhss, const float *rhss,
        float *lbs, float *ubs, const int *vartypes,
        const int sync_type GDP_DEFAULT_SYNC);

/* Replace reference include/interface.h:100-251 (CPU algorithms and research
 * measure variants). All return GDP_NOTIMPLEMENTED: no CPU fallback here. */
GDP_RETCODE propagateConstraintsSequentialDouble(
        const int n_cons, const int n_vars, const int nnz,
        const int *col_indices, const int *row_indices, const double *vals,
        const double *lhss, const double *rhss,
        double *lbs, double *ubs, const int *vartypes);

GDP_RETCODE propagateConstraintsSequentialFloat(
        const int n_cons, const int n_vars, const int nnz,
        const int *col_indices, const int *row_indices, const float *vals,
        const float *lhss, const float *rhss,
        float *lbs, float *ubs, const int *vartypes);

GDP_RETCODE propagateConstraintsFullOMPDouble(
        const int n_cons, const int n_vars, const int nnz,
        const int *col_indices, const int *row_indices, const double *vals,
        const double *lhss, const double *rhss,
        double *lbs, double *ubs, const int *vartypes);

GDP_RETCODE propagateConstraintsFullOMPFloat(
        const int n_cons, const int n_vars, const int nnz,
        const int *col_indices, const int *row_indices, const float *vals,
        const float *lhss, const float *rhss,
        float *lbs, float *ubs, const int *vartypes);

GDP_RETCODE propagateConstraintsSequentialDisjointDouble(
        const int n_cons, const int n_vars, const int nnz,
        const int *col_indices, const int *row_indices, const double *vals,
        const double *lhss, const double *rhss,
        double *lbs, double *ubs, const int *vartypes);

GDP_RETCODE sequentialPropagateWithMeasureDouble(
        const int n_cons, const int n_vars, const int nnz,
        const int *col_indices, const int *row_indices, const double *vals,
        const double *lhss, const double *rhss,
        double *lbs, double *ubs, const int *vartypes);

GDP_RETCODE atomicPropagateWithMeasureDouble(
        const int n_cons, const int n_vars, const int nnz,
        const int *col_indices, const int *row_indices, const double *vals,
        const double *lhss, const double *rhss,
        double *lbs, double *ubs, const int *vartypes);

#ifdef __cplusplus
}
#endif

#undef GDP_DEFAULT_SYNC

#endif /* GDP_GB300_INTERFACE_H */
