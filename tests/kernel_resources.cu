// The FP32 step's kernels for tracer groups of 4 (and of 2, the residual
// form's node kernels), instantiated alone so that
// tests/test_kernel_resources.py can read ptxas's register and spill report
// for them without compiling every launch variant of the library.
#include "fgb_fast_launch.cuh"

namespace fgb {
namespace fast {

// whole-column LO kernel, PPM vertical scheme: plain and compensated LO sums
template __global__ void kf_lo64<3, 4, false, false, false>(DMesh, FastPtrs);
template __global__ void kf_lo64<3, 4, false, false, true>(DMesh, FastPtrs);
// whole-column ratio kernel: lean and full
template __global__ void kf_ratio64<4, true, false>(DMesh, FastPtrs);
template __global__ void kf_ratio64<4, false, false>(DMesh, FastPtrs);
// update, one layer per lane: FP32 storage and with the rounding residual
template __global__ void kf_update<4, 1, false, false, false>(DMesh, FastPtrs);
template __global__ void kf_update<4, 1, false, false, true>(DMesh, FastPtrs);
// tiled edge-flux kernel, MUSCL and MFCT with FCT
template __global__ void kf_hflux_tile<1, true, 4>(DMesh, FastPtrs);
template __global__ void kf_hflux_tile<2, true, 4>(DMesh, FastPtrs);
// tracer groups of 2: LO with compensated sums, lean ratio, update with the residual
template __global__ void kf_lo64<3, 2, false, false, true>(DMesh, FastPtrs);
template __global__ void kf_ratio64<2, true, false>(DMesh, FastPtrs);
template __global__ void kf_update<2, 1, false, false, true>(DMesh, FastPtrs);

// the edge volume fluxes (a non-template kernel of internal linkage: its
// address keeps it in this unit)
void* keep_vflux() { return reinterpret_cast<void*>(&kf_vflux); }

}  // namespace fast
}  // namespace fgb
