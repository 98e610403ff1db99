// The fast-math instantiation of the DDA wavefront tracker
// (pt_wavefront_impl.cuh): built without -fmad=false and with VCR_FAST_MATH,
// so multiply-adds contract into FMAs and vlog / vexp / vsincos2pi use the
// hardware approximations.  Results are no longer bit-exact with the
// oracle; vcr_tuning.fast_math selects this kernel.
#ifndef VCR_FAST_MATH
#error "pt_wavefront_fast.cu is built with -DVCR_FAST_MATH"
#endif
#define VCR_WF_NS fast
#include "pt_wavefront_impl.cuh"
