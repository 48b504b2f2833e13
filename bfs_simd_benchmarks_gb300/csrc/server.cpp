// server.cpp -- the serving loop: resident graphs, admission by a device-
// memory budget, coalescing of the queries waiting on one graph into one
// batched traversal, continuous batching over a few in-flight result slots.
//
// No counterpart in the reference (one source per program run,
// apps/bfs_simd/bfs.cpp:1159).  Threads:
//   - the dispatcher takes, whenever a slot is free, the graph whose oldest
//     waiting query is oldest (among graphs with no batch in flight: a graph's
//     batch state serves one traversal at a time), moves up to its per-batch
//     capacity of waiting queries into the slot and enqueues the traversal on
//     the slot's stream; the traversal waits (by event) for the previous
//     traversal of any slot, so cooperative traversals never share the GPU,
//     while the previous batch's output pass and copies overlap this one;
//   - one worker per slot waits for its batch, copies host results, records
//     latencies and frees the slot and the graph.
// Result slots, streams and events are created with the server and every
// graph's batch state is reserved at admission, so no query allocates device
// memory.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/bfs_gb300.h"
#include "batch_hooks.h"
#include "msbfs.h"

namespace {

using Clock = std::chrono::steady_clock;

double ms_between(Clock::time_point a, Clock::time_point b) {
	return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Query {
	uint64_t ticket = 0;
	uint32_t source = 0;
	void *dst = nullptr;
	uint32_t dst_kind = BFS_DST_NONE;
	bool waitable = true;
	Clock::time_point t_submit, t_launch;
};

struct Record {
	bool done = false;
	bfs_query_result res{};
};

struct GraphEntry {
	bfs_graph *g = nullptr;
	uint32_t n = 0;
	uint32_t cap = 0;  // queries per traversal
	std::deque<Query> pending;
	bool in_flight = false;
	size_t bytes = 0;
};

struct Slot {
	int index = 0;
	cudaStream_t stream = nullptr;
	cudaEvent_t trav = nullptr;  // recorded after the traversal, before the output pass
	cudaEvent_t t0 = nullptr, done = nullptr;
	uint8_t *out = nullptr;
	std::thread worker;
	std::mutex mu;
	std::condition_variable cv;
	bool has_work = false;
	bool stop = false;
	// the batch it holds
	uint32_t graph = 0;
	int launch_status = BFS_OK;
	uint64_t batch_id = 0;
	std::vector<Query> queries;
};

size_t batch_state_estimate(uint32_t n, uint32_t K, uint32_t planes) {
	const size_t row = (size_t) n * K * 8;
	return row + (size_t) planes * (row + (size_t) n * 8) + (size_t) n * (2 + 4 + 8) + (1u << 16);
}

} // namespace

struct bfs_server {
	bfs_server_options opt{};
	int device = 0;
	std::mutex mu;  // everything below
	std::condition_variable cv_dispatch, cv_done;
	std::deque<GraphEntry> graphs;  // a deque: references stay valid as graphs are added
	std::vector<std::unique_ptr<Slot>> slots;
	std::vector<int> free_slots;
	std::unordered_map<uint64_t, Record> records;
	uint64_t next_ticket = 1, next_batch = 1;
	uint64_t pending_total = 0, inflight = 0;
	size_t used_bytes = 0;
	cudaEvent_t last_trav = nullptr;
	bool stop = false;
	std::thread dispatcher;
	// statistics since the last reset
	uint64_t submitted = 0, completed = 0, refused = 0, batches = 0, edges = 0, batch_queries = 0;
	double device_ms = 0;
	std::vector<float> lat_ms;
};

namespace {

void finish_batch(bfs_server *s, Slot &sl) {
	GraphEntry &ge = s->graphs[sl.graph];
	int status = sl.launch_status;
	bfs_batch_stats bst{};
	float dms = 0;
	if (status == BFS_OK) {
		if (cudaEventSynchronize(sl.done) != cudaSuccess) status = BFS_ECUDA;
	}
	if (status == BFS_OK) {
		status = bfs_last_batch_stats(ge.g, &bst);
		cudaEventElapsedTime(&dms, sl.t0, sl.done);
	}
	if (status == BFS_OK) {
		for (size_t i = 0; i < sl.queries.size(); ++i) {
			const Query &q = sl.queries[i];
			if (q.dst_kind != BFS_DST_HOST) continue;
			if (cudaMemcpyAsync(q.dst, sl.out + i * (size_t) ge.n, ge.n, cudaMemcpyDeviceToHost, sl.stream) != cudaSuccess) {
				status = BFS_ECUDA;
				break;
			}
		}
		if (cudaStreamSynchronize(sl.stream) != cudaSuccess) status = BFS_ECUDA;
	}
	const Clock::time_point t_done = Clock::now();
	std::lock_guard<std::mutex> lk(s->mu);
	for (const Query &q : sl.queries) {
		const double lat = ms_between(q.t_submit, t_done);
		s->lat_ms.push_back((float) lat);
		if (!q.waitable) continue;
		auto it = s->records.find(q.ticket);
		if (it == s->records.end()) continue;
		Record &r = it->second;
		r.res.status = status;
		r.res.batch_size = (uint32_t) sl.queries.size();
		r.res.batch_id = sl.batch_id;
		r.res.latency_ms = lat;
		r.res.queue_ms = ms_between(q.t_submit, q.t_launch);
		r.done = true;
	}
	s->completed += sl.queries.size();
	s->batches++;
	s->batch_queries += sl.queries.size();
	if (status == BFS_OK) s->edges += bst.edges_traversed;
	s->device_ms += dms;
	s->inflight -= sl.queries.size();
	sl.queries.clear();
	ge.in_flight = false;
	s->free_slots.push_back(sl.index);
	s->cv_dispatch.notify_one();
	s->cv_done.notify_all();
}

void slot_worker(bfs_server *s, Slot *sl) {
	cudaSetDevice(s->device);
	for (;;) {
		{
			std::unique_lock<std::mutex> lk(sl->mu);
			sl->cv.wait(lk, [&] { return sl->has_work || sl->stop; });
			if (!sl->has_work) return;
			// cleared before the slot is freed: the dispatcher may refill it at once
			sl->has_work = false;
		}
		finish_batch(s, *sl);
	}
}

// Index of the graph to serve next: the oldest waiting query among graphs
// with no batch in flight; -1 if none.
int pick_graph(const bfs_server *s) {
	int best = -1;
	for (size_t i = 0; i < s->graphs.size(); ++i) {
		const GraphEntry &ge = s->graphs[i];
		if (ge.in_flight || ge.pending.empty()) continue;
		if (best < 0 || ge.pending.front().t_submit < s->graphs[best].pending.front().t_submit) best = (int) i;
	}
	return best;
}

void dispatcher(bfs_server *s) {
	cudaSetDevice(s->device);
	std::unique_lock<std::mutex> lk(s->mu);
	for (;;) {
		int gi = -1;
		s->cv_dispatch.wait(lk, [&] { return s->stop || (!s->free_slots.empty() && (gi = pick_graph(s)) >= 0); });
		if (gi < 0) {
			if (s->stop) return;
			continue;
		}
		GraphEntry &ge = s->graphs[gi];
		const int si = s->free_slots.back();
		s->free_slots.pop_back();
		Slot &sl = *s->slots[si];
		const size_t nb = std::min<size_t>(ge.cap, ge.pending.size());
		sl.queries.assign(ge.pending.begin(), ge.pending.begin() + nb);
		ge.pending.erase(ge.pending.begin(), ge.pending.begin() + nb);
		ge.in_flight = true;
		s->pending_total -= nb;
		s->inflight += nb;
		sl.graph = (uint32_t) gi;
		sl.batch_id = s->next_batch++;
		cudaEvent_t wait = s->last_trav;
		s->last_trav = sl.trav;
		bfs_graph *g = ge.g;
		const uint32_t n = ge.n;
		lk.unlock();

		std::vector<uint32_t> src(nb);
		const Clock::time_point t_launch = Clock::now();
		for (size_t i = 0; i < nb; ++i) {
			src[i] = sl.queries[i].source;
			sl.queries[i].t_launch = t_launch;
		}
		int rc = cudaEventRecord(sl.t0, sl.stream) == cudaSuccess ? BFS_OK : BFS_ECUDA;
		if (rc == BFS_OK) rc = bfsg::run_batch_ex(g, src.data(), (uint32_t) nb, sl.out, sl.stream, wait, sl.trav);
		for (size_t i = 0; i < nb && rc == BFS_OK; ++i) {
			const Query &q = sl.queries[i];
			if (q.dst_kind == BFS_DST_DEVICE &&
					cudaMemcpyAsync(q.dst, sl.out + i * (size_t) n, n, cudaMemcpyDeviceToDevice, sl.stream) != cudaSuccess)
				rc = BFS_ECUDA;
		}
		if (rc == BFS_OK && cudaEventRecord(sl.done, sl.stream) != cudaSuccess) rc = BFS_ECUDA;
		{
			std::lock_guard<std::mutex> wl(sl.mu);
			sl.launch_status = rc;
			sl.has_work = true;
		}
		sl.cv.notify_one();
		lk.lock();
	}
}

int submit_locked(bfs_server *s, uint32_t graph_id, uint32_t source, void *dst, uint32_t dst_kind, bool waitable,
		uint64_t *ticket) {
	if (graph_id >= s->graphs.size()) return BFS_EARG;
	GraphEntry &ge = s->graphs[graph_id];
	if (source >= ge.n || dst_kind > BFS_DST_DEVICE || (dst_kind != BFS_DST_NONE && !dst)) return BFS_EARG;
	if (s->pending_total >= s->opt.max_pending) {
		s->refused++;
		return BFS_EBUDGET;
	}
	Query q;
	q.ticket = s->next_ticket++;
	q.source = source;
	q.dst = dst;
	q.dst_kind = dst_kind;
	q.waitable = waitable;
	q.t_submit = Clock::now();
	ge.pending.push_back(q);
	s->pending_total++;
	s->submitted++;
	if (waitable) s->records.emplace(q.ticket, Record{});
	if (ticket) *ticket = q.ticket;
	s->cv_dispatch.notify_one();
	return BFS_OK;
}

void release(bfs_server *s) {
	for (auto &sp : s->slots) {
		Slot &sl = *sp;
		if (sl.out) cudaFree(sl.out);
		if (sl.stream) cudaStreamDestroy(sl.stream);
		if (sl.trav) cudaEventDestroy(sl.trav);
		if (sl.t0) cudaEventDestroy(sl.t0);
		if (sl.done) cudaEventDestroy(sl.done);
	}
	s->slots.clear();
}

} // namespace

extern "C" {

int bfs_server_options_default(bfs_server_options *opt) {
	if (!opt) return BFS_EARG;
	std::memset(opt, 0, sizeof(*opt));
	opt->budget_bytes = (uint64_t) 40 << 30;
	opt->slot_bytes = (uint64_t) 2 << 30;
	opt->max_batch = 1024;
	opt->num_slots = 3;
	opt->planes = 8;
	opt->max_pending = 1u << 20;
	return BFS_OK;
}

int bfs_server_create(const bfs_server_options *opt, bfs_server **out) {
	if (!out) return BFS_EARG;
	*out = nullptr;
	bfs_server_options o;
	bfs_server_options_default(&o);
	if (opt) o = *opt;
	if (o.max_batch == 0 || o.max_batch > BFS_BATCH_MAX_SOURCES || o.num_slots == 0 || o.num_slots > 16 ||
			o.planes < 2 || o.planes > bfsg::kMsMaxLevel + 1 || o.slot_bytes == 0 || o.max_pending == 0)
		return BFS_EARG;
	if ((uint64_t) o.num_slots * o.slot_bytes > o.budget_bytes) return BFS_EBUDGET;
	int ndev = 0;
	if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
		cudaGetLastError();
		return BFS_ENODEV;
	}
	std::unique_ptr<bfs_server> s(new bfs_server());
	s->opt = o;
	if (cudaGetDevice(&s->device) != cudaSuccess) return BFS_ECUDA;
	for (uint32_t i = 0; i < o.num_slots; ++i) {
		std::unique_ptr<Slot> sl(new Slot());
		sl->index = (int) i;
		bool ok = cudaStreamCreateWithFlags(&sl->stream, cudaStreamNonBlocking) == cudaSuccess &&
				cudaEventCreateWithFlags(&sl->trav, cudaEventDisableTiming) == cudaSuccess &&
				cudaEventCreate(&sl->t0) == cudaSuccess &&
				cudaEventCreateWithFlags(&sl->done, cudaEventBlockingSync) == cudaSuccess;
		if (ok && cudaMalloc(&sl->out, o.slot_bytes) != cudaSuccess) {
			cudaGetLastError();
			s->slots.push_back(std::move(sl));
			release(s.get());
			return BFS_ENOMEM;
		}
		s->slots.push_back(std::move(sl));
		if (!ok) {
			release(s.get());
			return BFS_ECUDA;
		}
		s->free_slots.push_back((int) i);
	}
	s->used_bytes = (size_t) o.num_slots * o.slot_bytes;
	bfs_server *sp = s.get();
	for (auto &sl : s->slots) sl->worker = std::thread(slot_worker, sp, sl.get());
	s->dispatcher = std::thread(dispatcher, sp);
	*out = s.release();
	return BFS_OK;
}

int bfs_server_add_graph(bfs_server *s, bfs_graph *g, uint32_t *graph_id) {
	if (!s || !g) return BFS_EARG;
	if (!bfsg::graph_on_device(g)) return BFS_EUNSUPPORTED;
	if (bfsg::graph_device(g) != s->device) return BFS_EARG;
	const uint32_t n = bfsg::graph_num_vertices(g);
	const uint32_t cap = (uint32_t) std::min<uint64_t>(s->opt.max_batch, s->opt.slot_bytes / std::max<uint32_t>(n, 1));
	if (cap == 0) return BFS_EBUDGET;  // one result does not fit a slot
	const uint32_t K = (cap + 63) / 64;
	const size_t gbytes = bfsg::graph_device_bytes(g);
	{
		std::lock_guard<std::mutex> lk(s->mu);
		if (s->used_bytes + gbytes + batch_state_estimate(n, K, s->opt.planes) > s->opt.budget_bytes) return BFS_EBUDGET;
	}
	size_t bbytes = 0;
	int st = bfsg::batch_reserve(g, K, s->opt.planes, &bbytes);
	if (st) return st;
	std::lock_guard<std::mutex> lk(s->mu);
	GraphEntry ge;
	ge.g = g;
	ge.n = n;
	ge.cap = cap;
	ge.bytes = gbytes + bbytes;
	s->used_bytes += ge.bytes;
	s->graphs.push_back(std::move(ge));
	if (graph_id) *graph_id = (uint32_t) (s->graphs.size() - 1);
	return BFS_OK;
}

int bfs_server_submit(bfs_server *s, uint32_t graph_id, uint32_t source, void *dst, uint32_t dst_kind,
		uint64_t *ticket) {
	if (!s) return BFS_EARG;
	std::lock_guard<std::mutex> lk(s->mu);
	return submit_locked(s, graph_id, source, dst, dst_kind, true, ticket);
}

int bfs_server_wait(bfs_server *s, uint64_t ticket, bfs_query_result *result) {
	if (!s) return BFS_EARG;
	std::unique_lock<std::mutex> lk(s->mu);
	auto it = s->records.find(ticket);
	if (it == s->records.end()) return BFS_EARG;
	const Record *rec = &it->second;  // element addresses survive rehashing, iterators do not
	s->cv_done.wait(lk, [&] { return rec->done; });
	const bfs_query_result r = rec->res;
	s->records.erase(ticket);
	if (result) *result = r;
	return r.status;
}

int bfs_server_drain(bfs_server *s) {
	if (!s) return BFS_EARG;
	std::unique_lock<std::mutex> lk(s->mu);
	s->cv_done.wait(lk, [&] { return s->pending_total == 0 && s->inflight == 0; });
	return BFS_OK;
}

int bfs_server_replay(bfs_server *s, uint32_t count, const uint32_t *graph_ids, const uint32_t *sources,
		const uint64_t *arrival_ns) {
	if (!s || (count && (!graph_ids || !sources || !arrival_ns))) return BFS_EARG;
	int first_err = BFS_OK;
	const Clock::time_point t0 = Clock::now();
	for (uint32_t i = 0; i < count; ++i) {
		const Clock::time_point target = t0 + std::chrono::nanoseconds(arrival_ns[i]);
		for (;;) {
			const Clock::time_point now = Clock::now();
			if (now >= target) break;
			const auto left = target - now;
			if (left > std::chrono::microseconds(200)) std::this_thread::sleep_for(left - std::chrono::microseconds(100));
		}
		std::lock_guard<std::mutex> lk(s->mu);
		const int st = submit_locked(s, graph_ids[i], sources[i], nullptr, BFS_DST_NONE, false, nullptr);
		if (st && first_err == BFS_OK) first_err = st;
	}
	bfs_server_drain(s);
	return first_err;
}

int bfs_server_get_stats(bfs_server *s, bfs_server_stats *out) {
	if (!s || !out) return BFS_EARG;
	std::lock_guard<std::mutex> lk(s->mu);
	bfs_server_stats st{};
	st.submitted = s->submitted;
	st.completed = s->completed;
	st.refused = s->refused;
	st.batches = s->batches;
	st.edges_traversed = s->edges;
	st.device_ms = s->device_ms;
	st.device_bytes = s->used_bytes;
	st.graphs = (uint32_t) s->graphs.size();
	st.mean_batch = s->batches ? (double) s->batch_queries / s->batches : 0.0;
	if (!s->lat_ms.empty()) {
		std::vector<float> v = s->lat_ms;
		auto pct = [&](double p) {
			const size_t k = std::min(v.size() - 1, (size_t) (p * (v.size() - 1) + 0.5));
			std::nth_element(v.begin(), v.begin() + k, v.end());
			return (double) v[k];
		};
		st.p50_ms = pct(0.50);
		st.p99_ms = pct(0.99);
		double sum = 0, mx = 0;
		for (float x : s->lat_ms) {
			sum += x;
			mx = std::max(mx, (double) x);
		}
		st.mean_ms = sum / s->lat_ms.size();
		st.max_ms = mx;
	}
	*out = st;
	return BFS_OK;
}

int bfs_server_reset_stats(bfs_server *s) {
	if (!s) return BFS_EARG;
	std::lock_guard<std::mutex> lk(s->mu);
	s->submitted = s->completed = s->refused = s->batches = s->edges = s->batch_queries = 0;
	s->device_ms = 0;
	s->lat_ms.clear();
	return BFS_OK;
}

int bfs_server_destroy(bfs_server *s) {
	if (!s) return BFS_EARG;
	bfs_server_drain(s);
	{
		std::lock_guard<std::mutex> lk(s->mu);
		s->stop = true;
	}
	s->cv_dispatch.notify_all();
	if (s->dispatcher.joinable()) s->dispatcher.join();
	for (auto &sl : s->slots) {
		{
			std::lock_guard<std::mutex> lk(sl->mu);
			sl->stop = true;
		}
		sl->cv.notify_all();
		if (sl->worker.joinable()) sl->worker.join();
	}
	release(s);
	delete s;
	return BFS_OK;
}

} // extern "C"
