// Segmented sort kernels for 2-byte keys (one unit per key width, so the
// widths compile in parallel).
#include "seg_kernels.cuh"

namespace clo {
namespace seg {

template cudaError_t seg_launch_cta_classes<uint16_t>(const SegShape &, uint16_t *, const uint64_t *,
	const uint32_t *, const uint32_t *, uint32_t, int, uint64_t, CCLContext *, cudaStream_t);
template cudaError_t seg_launch_pass<uint16_t>(const SegShape &, const uint16_t *, uint16_t *,
	const SegPassArgs &, uint64_t, CCLContext *, cudaStream_t);

}  // namespace seg
}  // namespace clo
