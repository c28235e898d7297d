/*
 * gdp_types.h -- data contracts shared by the C API (interface.h) and the
 * extended API (gdp_ext.h) of the GB300 domain propagator.
 *
 * The enum names and numeric values are part of the binary interface that
 * existing callers of the reference library were compiled against, so they are
 * kept identical to the reference (src/def.h:15-20 GDP_Retcode, :29-34
 * GDP_Vartype, :42-47 GDP_Synctype; src/params.h:17-19 GDP_INF / GDP_EPS).
 */
#ifndef GDP_GB300_TYPES_H
#define GDP_GB300_TYPES_H

#ifdef __cplusplus
extern "C" {
#endif

/** Return codes: non-positive values are errors (reference src/def.h:15-20). */
enum GDP_Retcode {
    GDP_OKAY = +1,            /**< normal termination */
    GDP_ERROR = 0,            /**< unspecified error (message: gdp_last_error()) */
    GDP_NOTIMPLEMENTED = -18  /**< function not implemented by this library */
};
typedef enum GDP_Retcode GDP_RETCODE;

/** Variable types (reference src/def.h:29-34). Anything other than
 *  GDP_CONTINUOUS is integral and gets EPSFLOOR/EPSCEIL rounding. */
enum GDP_Vartype {
    GDP_BINARY = 0,
    GDP_INTEGER = 1,
    GDP_CONTINUOUS = 3
};
typedef enum GDP_Vartype GDP_VARTYPE;

/** Round-loop drivers (reference src/def.h:42-47).
 *  CPU_LOOP   : one launch group per round, host reads the change flag.
 *  GPU_LOOP   : device-driven loop -- here a CUDA graph with a conditional
 *               WHILE node (the reference used dynamic parallelism, which no
 *               longer exists in CUDA 12+).
 *  MEGAKERNEL : one persistent cooperative launch runs every round. */
enum GDP_Synctype {
    CPU_LOOP = 0,
    GPU_LOOP = 1,
    MEGAKERNEL = 2
};
typedef enum GDP_Synctype GDP_SYNCTYPE;

/** Bound magnitude treated as infinite (values >= GDP_INF are +inf). */
#define GDP_INF 1e20
/** Absolute comparison tolerance of every EPS test (reference src/params.h:19). */
#define GDP_EPS 1e-9
/** Relative feasibility tolerance of the infeasibility rule: a variable is
 *  infeasible when lb - ub > GDP_FEASTOL * max(1, |lb|, |ub|). The reference
 *  has no infeasibility detection on any propagation path; this rule is the
 *  one the oracle and the GPU path both apply after every round. */
#define GDP_FEASTOL 1e-6
/** Round cap of the reference (src/params.h:11). */
#define GDP_MAX_NUM_ROUNDS 100

#ifdef __cplusplus
}
#endif

#endif /* GDP_GB300_TYPES_H */
