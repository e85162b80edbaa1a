/*
 * TEST INFRASTRUCTURE -- fiber scheduler of clc_host.h (see there).
 */
#include "clc_host.h"

#include <ucontext.h>

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

size_t clc_local_id() { return clc_cur ? clc_cur->lid : 0; }

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

bool clc_run(size_t gws, size_t lws, const std::function<void()> &fn,
	const std::function<void()> &local_init) {
	if (lws == 0 || gws % lws) return false;
	const size_t kStack = 64 * 1024;
	std::vector<ClcWorkItem> wi(lws);
	std::vector<char> stacks(lws * kStack);
	clc_lsize = lws;
	clc_gsize = gws;
	clc_ngroups = gws / lws;
	clc_fn = &fn;
	bool ok = true;
	for (size_t g = 0; g < clc_ngroups && ok; ++g) {
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
			size_t done = 0, waiting = 0;
			for (size_t l = 0; l < lws; ++l) {
				ClcWorkItem &w = wi[l];
				if (w.done) continue;
				w.at_barrier = false;
				clc_cur = &w;
				swapcontext(&clc_sched, &w.ctx);
				if (w.done) ++done;
				else if (w.at_barrier) ++waiting;
			}
			size_t finished = 0;
			for (size_t l = 0; l < lws; ++l) finished += wi[l].done;
			if (finished == lws) break;
			if (finished != 0) {  /* some finished while others wait */
				ok = false;
				break;
			}
			(void)done;
			(void)waiting;
		}
	}
	clc_cur = nullptr;
	return ok;
}
