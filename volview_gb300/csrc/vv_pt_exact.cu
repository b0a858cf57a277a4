// vv_pt_exact.cu — the parity build of the single-path probe.
//
// Compiled with -DVV_EXACT=1 --fmad=false, once per density storage format,
// into namespace vv::exactN. Its samplers follow the texture-unit model the
// CPU oracle restates (texel coordinates through index_to_tex, decoded texels,
// the reference's folded B-spline fetches) and nothing is contracted into a
// fused multiply-add, so its arithmetic rounds as the oracle's does: the
// replays it runs differ from the oracle's only where CUDA's and the C
// library's expf/logf/powf/sinf/cosf/atan2f/acosf differ in the last bit. The
// product kernels (vv_pt.cu, vv_wavefront.cu) run the same code with the fast
// samplers and contraction; the tests compare them with this probe and with
// the oracle.
#include <cuda_runtime.h>

#include "vv_pt_device.cuh"

namespace vv {
namespace VV_FMT_NS {
#include "vv_pt_probe.cuh"
}  // namespace VV_FMT_NS
}  // namespace vv
