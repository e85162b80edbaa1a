// Optional per-kernel device-time accounting: when enabled, launchers
// bracket their kernels with CUDA events on the launching stream; totals
// are summed per kernel name on request. Off by default (no events).
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "clo_internal.h"
#include "timing.h"

namespace clo {
namespace {

struct Pending {
	std::string name;
	cudaEvent_t a, b;
	double bytes;
};

struct Totals {
	double ms = 0.0;
	double bytes = 0.0;
	unsigned long long launches = 0;
};

std::mutex g_mu;
bool g_on = false;
std::vector<Pending> g_pending;
std::map<std::string, Totals> g_totals;

void drain_locked() {
	for (Pending &p : g_pending) {
		cudaEventSynchronize(p.b);
		float ms = 0.f;
		if (cudaEventElapsedTime(&ms, p.a, p.b) == cudaSuccess) {
			Totals &t = g_totals[p.name];
			t.ms += ms;
			t.bytes += p.bytes;
			t.launches++;
		}
		cudaEventDestroy(p.a);
		cudaEventDestroy(p.b);
	}
	g_pending.clear();
}

}  // namespace

KernelTimer::KernelTimer(const char *name, cudaStream_t s, double bytes)
	: name_(name), s_(s), bytes_(bytes), a_(nullptr), b_(nullptr), on_(false) {
	std::lock_guard<std::mutex> lk(g_mu);
	if (!g_on || stream_capturing(s)) return;
	on_ = cudaEventCreate(&a_) == cudaSuccess && cudaEventCreate(&b_) == cudaSuccess;
	if (on_) cudaEventRecord(a_, s_);
}

void KernelTimer::stop() {
	if (!on_) return;
	cudaEventRecord(b_, s_);
	std::lock_guard<std::mutex> lk(g_mu);
	g_pending.push_back({name_, a_, b_, bytes_});
	on_ = false;
}

}  // namespace clo

extern "C" {

void clo_gb300_timing_enable(int on) {
	std::lock_guard<std::mutex> lk(clo::g_mu);
	clo::g_on = on != 0;
}

void clo_gb300_timing_reset(void) {
	std::lock_guard<std::mutex> lk(clo::g_mu);
	clo::drain_locked();
	clo::g_totals.clear();
}

int clo_gb300_timing_get(const char *kernel, double *total_ms,
	double *total_bytes, cl_ulong *launches) {
	std::lock_guard<std::mutex> lk(clo::g_mu);
	clo::drain_locked();
	auto it = clo::g_totals.find(kernel ? kernel : "");
	if (it == clo::g_totals.end()) return 0;
	if (total_ms) *total_ms = it->second.ms;
	if (total_bytes) *total_bytes = it->second.bytes;
	if (launches) *launches = it->second.launches;
	return 1;
}

}  // extern "C"
