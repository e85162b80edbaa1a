// Serving layer: admission by device-memory budget, continuous batching of
// small same-kind requests into segmented calls, several streams in
// flight, per-request latency.
//
// Threads: the caller(s) submit; one scheduler thread admits and launches
// batches (it is the only thread that enqueues device work); one
// completion thread per stream waits on its batches' events in launch
// order, stamps completion times and returns budget.
#include <algorithm>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include "clo_internal.h"
#include "clo_serve.h"

using clo::cuda_ok;
using clo::set_error;

namespace {

using Clock = std::chrono::steady_clock;

// Small requests (batched) and batch limits.
constexpr size_t kSmallN = 1u << 20;
constexpr size_t kBatchElems = 1u << 26;
constexpr size_t kMaxBatch = 4096;

double now_s() {
	return std::chrono::duration<double>(Clock::now().time_since_epoch()).count();
}

bool request_ok(const CloServeRequest *r) {
	if (!r) return false;
	switch (r->op) {
	case CLO_SERVE_SORT:
		return clo::type_is_integer(r->type) && r->n < (1u << 30) && (r->n == 0 || (r->in && r->out));
	case CLO_SERVE_SCAN:
		return clo::type_is_integer(r->type) && clo::type_is_integer(r->sum_type) &&
			r->n < (1u << 30) && (r->n == 0 || (r->in && r->out));
	case CLO_SERVE_RNG_FILL:
		return r->rng >= 0 && r->rng <= clo::RNG_TAUSLCG && r->draws > 0 &&
			(r->n == 0 || (r->in && r->out));
	}
	return false;
}

size_t elements_of(const CloServeRequest &r) {
	return r.op == CLO_SERVE_RNG_FILL ? r.n * r.draws : r.n;
}

struct Item {
	CloServeRequest r;
	uint64_t ticket;
	double t_submit = 0, t_done = 0;
	size_t bytes = 0;
	bool done = false;
	bool failed = false;
};

struct Batch {
	std::vector<Item *> items;
	size_t bytes = 0;
	cudaEvent_t ev_start = nullptr;  // recorded before the batch's first operation
	cudaEvent_t ev = nullptr;        // after its last
	// Pinned: kMaxBatch + 1 offsets of a segmented call, then (device-
	// resident batches) kMaxBatch input and kMaxBatch output pointers.
	uint64_t *h_off = nullptr;
	bool failed = false;
};

// Pinned words per batch buffer (offsets, input and output pointers).
constexpr size_t kPinnedWords = 3 * kMaxBatch + 1;

struct Lane {
	cudaStream_t stream = nullptr;
	std::mutex mu;
	std::condition_variable cv;
	std::deque<Batch *> q;
	std::thread th;
};

}  // namespace

struct clo_server {
	CCLContext *ctx;
	size_t budget;
	std::vector<Lane *> lanes;
	size_t next_lane = 0;

	std::mutex mu;
	std::condition_variable cv;
	std::deque<Item *> pending;
	std::unordered_map<uint64_t, Item *> items;
	uint64_t next_ticket = 1;
	size_t in_use = 0;
	size_t inflight = 0;   // admitted, not completed
	std::atomic<bool> stop{false};
	std::thread sched;

	std::vector<uint64_t *> pinned_free;  // kMaxBatch + 1 offsets each

	// batching policy (clo_serve_configure)
	size_t small_n = kSmallN, batch_elems = kBatchElems, max_batch = kMaxBatch;

	// Device clock origin: batches' start and end events are timed from
	// this event, so intervals of batches on different streams compare.
	cudaEvent_t origin = nullptr;

	// Batches' events come from and return to this pool, so that no driver
	// object is created or destroyed per batch.
	std::mutex ev_mu;
	std::vector<cudaEvent_t> ev_free;

	// statistics
	CloServeStats st;
	std::vector<double> lat_ms;
	std::vector<std::pair<double, double>> busy_ms;  // per batch [start, end]
	double t_first = 0, t_last = 0;
};

namespace {

size_t elem_bytes(CloType t) { return clo_type_sizeof(t); }

cudaEvent_t event_get(clo_server *srv) {
	{
		std::lock_guard<std::mutex> lk(srv->ev_mu);
		if (!srv->ev_free.empty()) {
			cudaEvent_t ev = srv->ev_free.back();
			srv->ev_free.pop_back();
			return ev;
		}
	}
	cudaEvent_t ev = nullptr;
	if (cudaEventCreate(&ev) != cudaSuccess) {
		cudaGetLastError();
		return nullptr;
	}
	return ev;
}

void event_put(clo_server *srv, cudaEvent_t ev) {
	if (!ev) return;
	std::lock_guard<std::mutex> lk(srv->ev_mu);
	srv->ev_free.push_back(ev);
}

void launch_batch(clo_server *srv, Batch *b, Lane *lane) {
	cudaStream_t s = lane->stream;
	b->ev_start = event_get(srv);
	if (b->ev_start) cudaEventRecord(b->ev_start, s);
	const CloServeRequest &r0 = b->items[0]->r;
	const bool dev_data = r0.device_data != CL_FALSE;
	const cudaMemcpyKind h2d = dev_data ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice;
	const cudaMemcpyKind d2h = dev_data ? cudaMemcpyDeviceToDevice : cudaMemcpyDeviceToHost;
	GError *err = nullptr;
	cudaError_t e = cudaSuccess;
	const size_t k = b->items.size();
	size_t total = 0;
	for (Item *it : b->items) total += it->r.n;
	if (r0.op == CLO_SERVE_RNG_FILL) {
		// The states are copied (the request's input is only read); the
		// draws go straight to a device-resident output.
		const size_t ss = clo_rng_infos[r0.rng].seed_size;
		const size_t draw_bytes = dev_data ? 0 : r0.n * r0.draws * 4;
		char *dev = (char *)clo::tmp_alloc(srv->ctx, r0.n * ss + draw_bytes + 256, s, &err);
		if (!dev) {
			b->failed = true;
		} else {
			char *states = dev;
			uint32_t *out = dev_data ? (uint32_t *)r0.out
				: (uint32_t *)(dev + (r0.n * ss + 255) / 256 * 256);
			e = cudaMemcpyAsync(states, r0.in, r0.n * ss, h2d, s);
			if (e == cudaSuccess)
				e = clo::rng_fill(states, r0.n, r0.rng, out, r0.draws, 32, 0, s);
			if (e == cudaSuccess && !dev_data)
				e = cudaMemcpyAsync(r0.out, out, r0.n * r0.draws * 4, d2h, s);
			clo::tmp_free(dev, s);
		}
	} else if (dev_data && k == 1) {
		// One device-resident request: the plain kernels on its buffers
		// (a sort copies its input to the output and sorts there).
		const size_t ib = elem_bytes(r0.type);
		const size_t ob = r0.op == CLO_SERVE_SCAN ? elem_bytes(r0.sum_type) : ib;
		if (r0.n && r0.op == CLO_SERVE_SORT) {
			if (r0.out != r0.in)
				e = cudaMemcpyAsync(r0.out, r0.in, r0.n * ib, cudaMemcpyDeviceToDevice, s);
			if (e == cudaSuccess)
				e = clo::radix_sort(r0.out, nullptr, r0.n, (int)ib, 0, (int)(8 * ib), srv->ctx,
					s, false, &err);
		} else if (r0.n) {
			e = clo::scan_exclusive(r0.in, r0.out, r0.n, r0.type, (int)ob, srv->ctx, s, &err);
		}
	} else {
		const size_t ib = elem_bytes(r0.type);
		const size_t ob = r0.op == CLO_SERVE_SCAN ? elem_bytes(r0.sum_type) : ib;
		uint64_t *h_off = b->h_off;
		h_off[0] = 0;
		for (size_t i = 0; i < k; ++i) h_off[i + 1] = h_off[i] + b->items[i]->r.n;
		// Device-resident batches also pass the requests' pointers.
		uint64_t *h_in = h_off + k + 1, *h_out = h_in + k;
		if (dev_data)
			for (size_t i = 0; i < k; ++i) {
				h_in[i] = (uint64_t)(uintptr_t)b->items[i]->r.in;
				h_out[i] = (uint64_t)(uintptr_t)b->items[i]->r.out;
			}
		// Device layout: [offsets (+ pointers)][inputs][outputs (scan)],
		// 256-byte aligned.
		const size_t meta_bytes = (dev_data ? 3 * k + 1 : k + 1) * 8;
		const size_t in_at = (meta_bytes + 255) / 256 * 256;
		const size_t out_at = r0.op == CLO_SERVE_SCAN ? (in_at + total * ib + 255) / 256 * 256
			: in_at;
		const size_t bytes = out_at + total * ob + 16;
		char *dev = (char *)clo::tmp_alloc(srv->ctx, bytes, s, &err);
		if (!dev) {
			b->failed = true;
		} else {
			uint64_t *d_off = (uint64_t *)dev;
			char *din = dev + in_at;
			char *dout = dev + out_at;
			e = cudaMemcpyAsync(d_off, h_off, meta_bytes, cudaMemcpyHostToDevice, s);
			if (dev_data) {
				if (e == cudaSuccess)
					e = clo::seg_gather(din, (const void *const *)(d_off + k + 1), d_off,
						(uint32_t)k, total, (int)ib, srv->ctx->sm_count, s);
			} else {
				for (size_t i = 0; i < k && e == cudaSuccess; ++i) {
					const CloServeRequest &r = b->items[i]->r;
					if (r.n)
						e = cudaMemcpyAsync(din + h_off[i] * ib, r.in, r.n * ib, h2d, s);
				}
			}
			if (e == cudaSuccess && total > 0) {
				// A request alone takes the plain kernels (the onesweep
				// sort, without the host readback of pass skipping);
				// a batch takes one segmented call.
				if (r0.op == CLO_SERVE_SORT && k == 1)
					e = clo::radix_sort(din, nullptr, total, (int)ib, 0, (int)(8 * ib),
						srv->ctx, s, false, &err);
				else if (r0.op == CLO_SERVE_SORT)
					e = clo::seg_sort(din, total, d_off, k, (int)ib, (int)(8 * ib), 0,
						srv->ctx, s, &err);
				else if (k == 1)
					e = clo::scan_exclusive(din, dout, total, r0.type, (int)ob, srv->ctx, s,
						&err);
				else
					e = clo::seg_scan(din, dout, total, d_off, k, r0.type, (int)ob,
						srv->ctx, s, &err);
			}
			if (dev_data) {
				if (e == cudaSuccess)
					e = clo::seg_scatter((void *const *)(d_off + 2 * k + 1), dout, d_off,
						(uint32_t)k, total, (int)ob, srv->ctx->sm_count, s);
			} else {
				for (size_t i = 0; i < k && e == cudaSuccess; ++i) {
					const CloServeRequest &r = b->items[i]->r;
					if (r.n)
						e = cudaMemcpyAsync(r.out, dout + h_off[i] * ob, r.n * ob, d2h, s);
				}
			}
			clo::tmp_free(dev, s);
		}
	}
	if (e != cudaSuccess) {
		cudaGetLastError();
		b->failed = true;
	}
	if (err) clo_error_free(err);
	b->ev = event_get(srv);
	if (b->ev) cudaEventRecord(b->ev, s);
}

void lane_loop(clo_server *srv, Lane *lane) {
	cudaSetDevice(srv->ctx->ordinal);
	for (;;) {
		Batch *b = nullptr;
		{
			std::unique_lock<std::mutex> lk(lane->mu);
			lane->cv.wait(lk, [&] { return !lane->q.empty() || srv->stop; });
			if (lane->q.empty()) return;
			b = lane->q.front();
			lane->q.pop_front();
		}
		bool failed = b->failed || !b->ev;
		if (b->ev) {
			if (cudaEventSynchronize(b->ev) != cudaSuccess) {
				cudaGetLastError();
				failed = true;
			}
		} else {
			cudaStreamSynchronize(lane->stream);
		}
		const double t = now_s();
		float t0_ms = 0.f, t1_ms = 0.f;
		const bool timed = b->ev_start && b->ev &&
			cudaEventElapsedTime(&t0_ms, srv->origin, b->ev_start) == cudaSuccess &&
			cudaEventElapsedTime(&t1_ms, srv->origin, b->ev) == cudaSuccess;
		if (!timed) cudaGetLastError();
		event_put(srv, b->ev_start);
		event_put(srv, b->ev);
		{
			std::lock_guard<std::mutex> lk(srv->mu);
			if (timed) srv->busy_ms.emplace_back((double)t0_ms, (double)t1_ms);
			for (Item *it : b->items) {
				it->done = true;
				it->failed = failed;
				it->t_done = t;
				if (failed) {
					srv->st.failed++;
				} else {
					srv->st.completed++;
					srv->lat_ms.push_back((t - it->t_submit) * 1e3);
					srv->st.elements += (double)elements_of(it->r);
				}
			}
			srv->t_last = t;
			srv->in_use -= b->bytes;
			srv->inflight -= b->items.size();
			if (b->h_off) srv->pinned_free.push_back(b->h_off);
		}
		srv->cv.notify_all();
		delete b;
	}
}

void sched_loop(clo_server *srv) {
	cudaSetDevice(srv->ctx->ordinal);
	std::vector<CloServeRequest> view;
	std::vector<size_t> chosen(kMaxBatch);
	for (;;) {
		Batch *b = new Batch();
		{
			std::unique_lock<std::mutex> lk(srv->mu);
			size_t k = 0;
			for (;;) {
				if (!srv->pending.empty()) {
					view.clear();
					const size_t look = std::min<size_t>(srv->pending.size(), 4 * kMaxBatch);
					for (size_t i = 0; i < look; ++i) view.push_back(srv->pending[i]->r);
					k = clo_serve_select(view.data(), view.size(), srv->budget - srv->in_use,
						srv->small_n, srv->batch_elems, srv->max_batch, chosen.data());
					if (k > 0) break;
				}
				if (srv->stop && srv->pending.empty()) {
					delete b;
					return;
				}
				srv->cv.wait(lk);
			}
			// Take the chosen requests out of the queue (indices ascend).
			std::vector<Item *> rest;
			size_t c = 0;
			for (size_t i = 0; i < srv->pending.size(); ++i) {
				if (c < k && chosen[c] == i) {
					b->items.push_back(srv->pending[i]);
					b->bytes += srv->pending[i]->bytes;
					++c;
				}
			}
			size_t w = 0;
			c = 0;
			for (size_t i = 0; i < srv->pending.size(); ++i) {
				if (c < k && chosen[c] == i) {
					++c;
					continue;
				}
				srv->pending[w++] = srv->pending[i];
			}
			srv->pending.resize(w);
			srv->in_use += b->bytes;
			srv->inflight += k;
			srv->st.peak_bytes = std::max(srv->st.peak_bytes, srv->in_use);
			srv->st.admitted += k;
			srv->st.batches++;
			if (b->items[0]->r.op != CLO_SERVE_RNG_FILL) {
				if (srv->pinned_free.empty()) {
					uint64_t *p = nullptr;
					if (cudaMallocHost(&p, kPinnedWords * 8) != cudaSuccess) {
						cudaGetLastError();
						p = nullptr;
					}
					if (p) srv->pinned_free.push_back(p);
				}
				if (!srv->pinned_free.empty()) {
					b->h_off = srv->pinned_free.back();
					srv->pinned_free.pop_back();
				}
			}
		}
		Lane *lane = srv->lanes[srv->next_lane++ % srv->lanes.size()];
		if (b->items[0]->r.op != CLO_SERVE_RNG_FILL && b->h_off == nullptr) {
			b->failed = true;
			b->ev = event_get(srv);
			if (b->ev) cudaEventRecord(b->ev, lane->stream);
		} else {
			launch_batch(srv, b, lane);
		}
		{
			std::lock_guard<std::mutex> lk(lane->mu);
			lane->q.push_back(b);
		}
		lane->cv.notify_one();
	}
}

}  // namespace

extern "C" {

size_t clo_serve_footprint(const CloServeRequest *r) {
	if (!request_ok(r)) return 0;
	const size_t slack = 1u << 20;  // tile statuses, offsets, alignment
	switch (r->op) {
	case CLO_SERVE_SORT: {
		// keys + the alternate key buffer of the passes + per-tile state:
		// two 1 KB lookback status slots and 28 B of segment descriptors
		// for every tile of at least 8192 keys (the smallest tile of a
		// keys-only pass)
		const size_t eb = elem_bytes(r->type);
		return 2 * r->n * eb + (r->n + 8191) / 8192 * 2076 + slack;
	}
	case CLO_SERVE_SCAN:
		return r->n * (elem_bytes(r->type) + elem_bytes(r->sum_type)) + r->n / 8 + slack;
	case CLO_SERVE_RNG_FILL:
		return r->n * clo_rng_infos[r->rng].seed_size + r->n * r->draws * 4 + slack;
	}
	return 0;
}

size_t clo_serve_select(const CloServeRequest *pending, size_t npending,
	size_t free_bytes, size_t small_n, size_t batch_elems, size_t max_batch,
	size_t *chosen) {
	if (npending == 0 || max_batch == 0 || !chosen) return 0;
	const CloServeRequest &h = pending[0];
	size_t need = clo_serve_footprint(&h);
	if (need == 0 || need > free_bytes) return 0;
	chosen[0] = 0;
	size_t k = 1;
	if (h.op == CLO_SERVE_RNG_FILL || h.n > small_n) return k;
	size_t elems = h.n;
	for (size_t i = 1; i < npending && k < max_batch; ++i) {
		const CloServeRequest &r = pending[i];
		if (r.op != h.op || r.type != h.type || r.n > small_n) continue;
		if ((r.device_data != CL_FALSE) != (h.device_data != CL_FALSE)) continue;
		if (h.op == CLO_SERVE_SCAN && r.sum_type != h.sum_type) continue;
		const size_t f = clo_serve_footprint(&r);
		if (f == 0 || elems + r.n > batch_elems || need + f > free_bytes) continue;
		need += f;
		elems += r.n;
		chosen[k++] = i;
	}
	return k;
}

CloServer *clo_serve_new(CCLContext *ctx, size_t budget_bytes, int streams, GError **err) {
	if (!ctx || streams < 1 || streams > 16 || budget_bytes == 0) {
		set_error(err, CLO_ERROR_ARGS, "clo_serve_new: a context, a budget and 1..16 streams");
		return nullptr;
	}
	cudaSetDevice(ctx->ordinal);
	clo_server *srv = new clo_server();
	srv->ctx = ctx;
	srv->budget = budget_bytes;
	memset(&srv->st, 0, sizeof srv->st);
	srv->st.budget_bytes = budget_bytes;
	ccl_context_ref(ctx);
	clo::wrapper_created();
	for (int i = 0; i < streams; ++i) {
		Lane *l = new Lane();
		if (!cuda_ok(cudaStreamCreateWithFlags(&l->stream, cudaStreamNonBlocking), err,
				"cudaStreamCreate")) {
			delete l;
			clo_serve_destroy(srv);
			return nullptr;
		}
		srv->lanes.push_back(l);
	}
	if (!cuda_ok(cudaEventCreate(&srv->origin), err, "cudaEventCreate") ||
		!cuda_ok(cudaEventRecord(srv->origin, srv->lanes[0]->stream), err, "cudaEventRecord") ||
		!cuda_ok(cudaEventSynchronize(srv->origin), err, "cudaEventSynchronize")) {
		clo_serve_destroy(srv);
		return nullptr;
	}
	for (Lane *l : srv->lanes) l->th = std::thread(lane_loop, srv, l);
	srv->sched = std::thread(sched_loop, srv);
	return srv;
}

cl_ulong clo_serve_submit(CloServer *srv, const CloServeRequest *req, GError **err) {
	if (!srv || (err && *err)) return 0;
	const size_t f = clo_serve_footprint(req);
	if (f == 0 || f > srv->budget) {
		std::lock_guard<std::mutex> lk(srv->mu);
		srv->st.rejected++;
		if (f == 0)
			set_error(err, CLO_ERROR_ARGS, "Malformed serving request");
		else
			set_error(err, CLO_ERROR_ARGS,
				"Request needs %zu device bytes, more than the server's budget of %zu",
				f, srv->budget);
		return 0;
	}
	Item *it = new Item();
	it->r = *req;
	it->bytes = f;
	it->t_submit = now_s();
	uint64_t t;
	{
		std::lock_guard<std::mutex> lk(srv->mu);
		t = it->ticket = srv->next_ticket++;
		srv->items[t] = it;
		srv->pending.push_back(it);
		srv->st.submitted++;
		if (srv->t_first == 0) srv->t_first = it->t_submit;
		srv->st.max_queued = std::max<cl_ulong>(srv->st.max_queued, srv->pending.size());
	}
	srv->cv.notify_all();
	return t;
}

cl_bool clo_serve_wait(CloServer *srv, cl_ulong ticket, double *latency_ms, GError **err) {
	if (!srv || (err && *err)) return CL_FALSE;
	std::unique_lock<std::mutex> lk(srv->mu);
	auto f = srv->items.find(ticket);
	if (f == srv->items.end()) {
		set_error(err, CLO_ERROR_ARGS, "Unknown ticket %llu", (unsigned long long)ticket);
		return CL_FALSE;
	}
	Item *it = f->second;
	srv->cv.wait(lk, [&] { return it->done; });
	if (latency_ms) *latency_ms = (it->t_done - it->t_submit) * 1e3;
	const bool failed = it->failed;
	srv->items.erase(f);
	delete it;
	if (failed) {
		set_error(err, CLO_ERROR_LIBRARY, "Serving request %llu failed on the device",
			(unsigned long long)ticket);
		return CL_FALSE;
	}
	return CL_TRUE;
}

cl_bool clo_serve_drain(CloServer *srv, GError **err) {
	if (!srv || (err && *err)) return CL_FALSE;
	{
		std::unique_lock<std::mutex> lk(srv->mu);
		srv->cv.wait(lk, [&] { return srv->pending.empty() && srv->inflight == 0; });
	}
	if (!clo::check_device_status(srv->ctx, err)) return CL_FALSE;
	std::lock_guard<std::mutex> lk(srv->mu);
	if (srv->st.failed) {
		set_error(err, CLO_ERROR_LIBRARY, "%llu serving request(s) failed on the device",
			(unsigned long long)srv->st.failed);
		return CL_FALSE;
	}
	return CL_TRUE;
}

cl_bool clo_serve_replay(CloServer *srv, const CloServeRequest *reqs,
	const double *arrival_s, size_t count, cl_ulong *tickets, GError **err) {
	if (!srv || (count && (!reqs || !arrival_s)) || (err && *err)) {
		set_error(err, CLO_ERROR_ARGS, "clo_serve_replay: bad arguments");
		return CL_FALSE;
	}
	const auto t0 = Clock::now();
	for (size_t i = 0; i < count; ++i) {
		const auto target = t0 + std::chrono::duration_cast<Clock::duration>(
			std::chrono::duration<double>(arrival_s[i]));
		for (;;) {
			const auto now = Clock::now();
			if (now >= target) break;
			if (target - now > std::chrono::microseconds(200))
				std::this_thread::sleep_for(std::chrono::microseconds(100));
		}
		GError *e2 = nullptr;
		const cl_ulong t = clo_serve_submit(srv, reqs + i, &e2);
		if (e2) clo_error_free(e2);
		if (tickets) tickets[i] = t;
	}
	return CL_TRUE;
}

cl_bool clo_serve_configure(CloServer *srv, size_t small_n, size_t batch_elems,
	size_t max_batch, GError **err) {
	if (!srv || (err && *err)) return CL_FALSE;
	if (max_batch < 1 || max_batch > kMaxBatch || batch_elems == 0) {
		set_error(err, CLO_ERROR_ARGS,
			"clo_serve_configure: max_batch must be 1..%zu and batch_elems nonzero", kMaxBatch);
		return CL_FALSE;
	}
	std::lock_guard<std::mutex> lk(srv->mu);
	srv->small_n = small_n;
	srv->batch_elems = batch_elems;
	srv->max_batch = max_batch;
	return CL_TRUE;
}

void clo_serve_get_stats(CloServer *srv, CloServeStats *out) {
	if (!srv || !out) return;
	std::vector<double> l;
	std::vector<std::pair<double, double>> busy;
	{
		std::lock_guard<std::mutex> lk(srv->mu);
		*out = srv->st;
		l = srv->lat_ms;
		busy = srv->busy_ms;
		out->span_s = srv->t_last > srv->t_first ? srv->t_last - srv->t_first : 0.0;
	}
	// Batches in flight on the device at once: a sweep over the batches'
	// [start, end] device intervals. The mean is the batches' summed device
	// time over the time at least one was in flight.
	if (!busy.empty()) {
		std::vector<std::pair<double, int>> ev;
		ev.reserve(2 * busy.size());
		double sum = 0;
		for (auto &iv : busy) {
			ev.emplace_back(iv.first, +1);
			ev.emplace_back(iv.second, -1);
			sum += iv.second - iv.first;
		}
		std::sort(ev.begin(), ev.end(), [](const std::pair<double, int> &a,
			const std::pair<double, int> &b) {
			return a.first < b.first || (a.first == b.first && a.second < b.second);
		});
		int cur = 0, peak = 0;
		double union_ms = 0, last = ev[0].first;
		for (auto &e : ev) {
			if (cur > 0) union_ms += e.first - last;
			last = e.first;
			cur += e.second;
			peak = std::max(peak, cur);
		}
		out->max_concurrent_batches = (cl_ulong)peak;
		out->device_busy_s = union_ms * 1e-3;
		out->mean_concurrent_batches = union_ms > 0 ? sum / union_ms : 0.0;
	}
	if (!l.empty()) {
		std::sort(l.begin(), l.end());
		auto pct = [&](double p) {
			size_t i = (size_t)(p * (double)(l.size() - 1) + 0.5);
			return l[std::min(i, l.size() - 1)];
		};
		out->p50_ms = pct(0.50);
		out->p99_ms = pct(0.99);
		out->max_ms = l.back();
		double s = 0;
		for (double v : l) s += v;
		out->mean_ms = s / (double)l.size();
	}
}

void clo_serve_reset_stats(CloServer *srv) {
	if (!srv) return;
	std::lock_guard<std::mutex> lk(srv->mu);
	const size_t budget = srv->st.budget_bytes;
	memset(&srv->st, 0, sizeof srv->st);
	srv->st.budget_bytes = budget;
	srv->lat_ms.clear();
	srv->busy_ms.clear();
	srv->t_first = srv->t_last = 0;
}

void clo_serve_destroy(CloServer *srv) {
	if (!srv) return;
	{
		std::unique_lock<std::mutex> lk(srv->mu);
		srv->cv.wait(lk, [&] { return srv->pending.empty() && srv->inflight == 0; });
		srv->stop = true;
	}
	srv->cv.notify_all();
	if (srv->sched.joinable()) srv->sched.join();
	for (Lane *l : srv->lanes) {
		{
			std::lock_guard<std::mutex> lk(l->mu);
		}
		l->cv.notify_all();
		if (l->th.joinable()) l->th.join();
	}
	cudaSetDevice(srv->ctx->ordinal);
	for (Lane *l : srv->lanes) {
		if (l->stream) cudaStreamDestroy(l->stream);
		delete l;
	}
	if (srv->origin) cudaEventDestroy(srv->origin);
	for (cudaEvent_t ev : srv->ev_free) cudaEventDestroy(ev);
	for (uint64_t *p : srv->pinned_free) cudaFreeHost(p);
	for (auto &kv : srv->items) delete kv.second;
	ccl_context_unref(srv->ctx);
	clo::wrapper_destroyed();
	delete srv;
}

}  // extern "C"
