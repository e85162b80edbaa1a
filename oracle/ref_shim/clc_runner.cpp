/*
 * TEST INFRASTRUCTURE -- fiber scheduler of clc_host.h (see there).
 *
 * Each worker thread runs whole work-groups, one at a time: a group's
 * work-items are ucontext fibers that the worker resumes in local-id order,
 * one barrier interval per round. Groups are taken from a shared counter,
 * so any number of workers gives the same results for kernels whose
 * work-groups are independent (all OpenCL kernels are).
 */
#include "clc_host.h"

#include <ucontext.h>

#include <atomic>
#include <cstdlib>
#include <thread>
#include <vector>

struct ClcWorkItem {
	ucontext_t ctx;
	size_t lid;
	bool done;
	bool at_barrier;
};

thread_local ClcWorkItem *clc_cur = nullptr;
thread_local size_t clc_group = 0, clc_lsize = 1, clc_gsize = 1, clc_ngroups = 1;
static thread_local ucontext_t clc_sched;
static thread_local const std::function<void()> *clc_fn = nullptr;
static thread_local size_t clc_worker_id = 0;

size_t clc_local_id() { return clc_cur ? clc_cur->lid : 0; }
size_t clc_worker() { return clc_worker_id; }

size_t clc_workers() {
	static const size_t n = [] {
		const char *e = getenv("CLC_THREADS");
		long v = e ? atol(e) : 0;
		if (v <= 0) v = (long)std::thread::hardware_concurrency();
		return (size_t)(v > 0 ? v : 1);
	}();
	return n;
}

void barrier(int flags) {
	(void)flags;
	clc_cur->at_barrier = true;
	swapcontext(&clc_cur->ctx, &clc_sched);
}

static void trampoline() {
	(*clc_fn)();
	clc_cur->done = true;
	/* uc_link returns to the scheduler */
}

/* Runs the groups this worker claims; false if a group's work-items
 * disagreed on barriers. */
static bool run_groups(size_t worker, size_t gws, size_t lws, const std::function<void()> &fn,
	const std::function<void()> &local_init, std::atomic<size_t> &next,
	std::atomic<bool> &failed) {
	const size_t kStack = 64 * 1024;
	std::vector<ClcWorkItem> wi(lws);
	std::vector<char> stacks(lws * kStack);
	clc_worker_id = worker;
	clc_lsize = lws;
	clc_gsize = gws;
	clc_ngroups = gws / lws;
	clc_fn = &fn;
	bool ok = true;
	for (size_t g = next.fetch_add(1); g < clc_ngroups && ok && !failed.load();
		 g = next.fetch_add(1)) {
		clc_group = g;
		if (local_init) local_init();
		for (size_t l = 0; l < lws; ++l) {
			ClcWorkItem &w = wi[l];
			w.lid = l;
			w.done = false;
			w.at_barrier = false;
			getcontext(&w.ctx);
			w.ctx.uc_stack.ss_sp = &stacks[l * kStack];
			w.ctx.uc_stack.ss_size = kStack;
			w.ctx.uc_link = &clc_sched;
			makecontext(&w.ctx, trampoline, 0);
		}
		for (;;) {
			for (size_t l = 0; l < lws; ++l) {
				ClcWorkItem &w = wi[l];
				if (w.done) continue;
				w.at_barrier = false;
				clc_cur = &w;
				swapcontext(&clc_sched, &w.ctx);
			}
			size_t finished = 0;
			for (size_t l = 0; l < lws; ++l) finished += wi[l].done;
			if (finished == lws) break;
			if (finished != 0) { /* some finished while others wait */
				ok = false;
				break;
			}
		}
	}
	clc_cur = nullptr;
	clc_worker_id = 0;
	if (!ok) failed.store(true);
	return ok;
}

bool clc_run(size_t gws, size_t lws, const std::function<void()> &fn,
	const std::function<void()> &local_init) {
	if (lws == 0 || gws % lws) return false;
	const size_t groups = gws / lws;
	size_t workers = clc_workers();
	if (workers > groups) workers = groups;
	std::atomic<size_t> next{0};
	std::atomic<bool> failed{false};
	if (workers <= 1) {
		run_groups(0, gws, lws, fn, local_init, next, failed);
		return !failed.load();
	}
	std::vector<std::thread> th;
	th.reserve(workers - 1);
	for (size_t w = 1; w < workers; ++w)
		th.emplace_back([&, w] { run_groups(w, gws, lws, fn, local_init, next, failed); });
	run_groups(0, gws, lws, fn, local_init, next, failed);
	for (auto &t : th) t.join();
	return !failed.load();
}
