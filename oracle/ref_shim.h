/*
 * ref_shim.h -- TEST INFRASTRUCTURE ONLY. Force-included (g++ -include) when
 * oracle/Makefile compiles the reference's CPU propagators host-only, so that
 * its headers build without CUDA device code or cuSPARSE:
 *   - the reference's CUDA utility header (src/kernels/util_kernels.cuh) is
 *     skipped by defining its include guard on the command line;
 *   - the reference's canConsBeTightened calls an unqualified min();
 *   - src/cuda_def.cuh needs the cudaError_t declarations only.
 */
#ifndef GDP_REF_SHIM_H
#define GDP_REF_SHIM_H
#include <algorithm>
#include <cassert>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <stdexcept>
#include <cuda_runtime_api.h>
using std::min;
using std::max;
#endif
