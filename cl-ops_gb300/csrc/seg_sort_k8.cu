// Segmented sort kernels for 8-byte keys (one unit per key width, so the
// widths compile in parallel).
#include "seg_kernels.cuh"

namespace clo {
namespace seg {

template cudaError_t seg_launch_cta_classes<uint64_t>(const SegShape &, uint64_t *, const uint64_t *,
	const uint32_t *, const uint32_t *, uint32_t, int, uint64_t, CCLContext *, cudaStream_t);
template cudaError_t seg_launch_pass<uint64_t>(const SegShape &, const uint64_t *, uint64_t *,
	const SegPassArgs &, uint64_t, CCLContext *, cudaStream_t);

}  // namespace seg
}  // namespace clo
