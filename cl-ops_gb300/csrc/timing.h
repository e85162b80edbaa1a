// Scoped kernel timer used by the launchers (see timing.cpp).
#pragma once

#include <cuda_runtime.h>

namespace clo {

class KernelTimer {
public:
	// `bytes` is the launch's algorithmic HBM traffic, summed alongside.
	KernelTimer(const char *name, cudaStream_t s, double bytes);
	void stop();

private:
	const char *name_;
	cudaStream_t s_;
	double bytes_;
	cudaEvent_t a_, b_;
	bool on_;
};

}  // namespace clo
