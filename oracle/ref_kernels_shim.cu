// ref_kernels_shim.cu -- TEST INFRASTRUCTURE.  Instantiates the reference
// project's own step-1/2/3 kernels (src/spgemm_raw_kernels.cuh,
// src/spgemm_raw_kernels_v2.cuh) into a cubin for sm_103a, compiled from the
// reference checkout where it lies (oracle/build_ref.sh).  The cubin is loaded
// through the CUDA driver API by tests/golden/make_cstruct_golden.py, which
// drives the kernels the way src/spgemm_raw_v2.cu:111-243 does and records
// C's tile arrays as golden fixtures.  Nothing of the reference is copied here.
// Include order as in src/spgemm_raw_v2.cu:3-11 (CUB before tile_format.h,
// whose TILE_SIZE macro would otherwise clash with a CUB member name).
#include <cub/cub.cuh>
#include "tile_format.h"
#include "spgemm_raw_kernels_v2.cuh"
