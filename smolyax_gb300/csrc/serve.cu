// Request queue of the serving path behind the C ABI (smx_serve_*).
//
// A host program submits FP32 evaluations of one-output plans (smx_blocked)
// and per-point plans (smx_spectral); each flush merges the queued requests of
// each kind into one persistent multi-plan launch (smx_blocked_eval_batch /
// smx_spectral_eval_batch: the blocks take 128-point tiles of any request from
// a shared counter, and every tile is evaluated exactly as alone) on the
// server's stream, and records an event.  Tickets are numbered in submission
// order; a flush covers a contiguous range of them, and flushes complete in
// order, so a ticket is done once the event of its flush has fired.  The
// workspaces of the launches in flight are allocated when the server is
// created (max_inflight flushes of up to max_items requests over up to
// max_plans plans per kind), so submitting and flushing allocate nothing.
#include <algorithm>
#include <deque>
#include <vector>

#include "common.cuh"

namespace {

struct Flight {
  int slot;             // index of the workspace pair in use
  int64_t end;          // tickets below this are done when the event fires
  cudaEvent_t event;
};

struct Failed {
  int64_t begin, end;   // tickets of a flush whose launch was refused or failed
  int rc;               // its error code, returned by smx_serve_poll
};

template <typename Plan>
struct Queue {
  std::vector<Plan> plans;           // copies of the distinct plans
  std::vector<const Plan*> keys;     // the caller's plan pointers (identity)
  std::vector<smx_work> items;
  int add_plan(const Plan* p) {
    for (size_t i = 0; i < keys.size(); ++i)
      if (keys[i] == p) return int(i);
    keys.push_back(p);
    plans.push_back(*p);
    return int(keys.size() - 1);
  }
  void clear() {
    plans.clear();
    keys.clear();
    items.clear();
  }
};

}  // namespace

struct smx_server {
  cudaStream_t stream = nullptr;
  int max_items = 0, max_plans = 0, max_inflight = 0;
  size_t ws_blocked = 0, ws_spectral = 0;
  std::vector<void*> ws;  // [max_inflight][2]: blocked, spectral
  std::vector<char> slot_busy;
  std::vector<cudaEvent_t> events;
  std::deque<Flight> flights;
  std::vector<Failed> failed;
  Queue<smx_blocked> blocked;
  Queue<smx_spectral> spectral;
  int64_t next_ticket = 0;   // tickets issued
  int64_t flushed_end = 0;   // tickets below this have been launched
  int64_t retired_end = 0;   // tickets below this are done
};

namespace {

// Pops the flights whose events have fired (they complete in stream order).
int retire(smx_server* s) {
  while (!s->flights.empty()) {
    const Flight& f = s->flights.front();
    const cudaError_t e = cudaEventQuery(f.event);
    if (e == cudaErrorNotReady) break;
    if (e != cudaSuccess) return smx::set_error(SMX_ERR_CUDA, "smx_serve: a batch launch failed");
    s->retired_end = f.end;
    s->slot_busy[f.slot] = 0;
    s->flights.pop_front();
  }
  return SMX_OK;
}

}  // namespace

extern "C" int smx_serve_create(int max_items, int max_plans, int max_inflight, void* stream, smx_server** out) {
  SMX_REQUIRE(out && max_items >= 1 && max_plans >= 1 && max_inflight >= 1 && max_inflight <= 64,
              "smx_serve_create: bad arguments");
  *out = nullptr;
  smx_server* s = new smx_server;
  s->stream = smx::as_stream(stream);
  s->max_items = max_items;
  s->max_plans = max_plans;
  s->max_inflight = max_inflight;
  s->ws_blocked = smx_blocked_eval_batch_workspace(max_plans, max_items);
  s->ws_spectral = smx_spectral_eval_batch_workspace(max_plans, max_items, 16);
  s->ws.assign(size_t(2) * max_inflight, nullptr);
  s->slot_busy.assign(max_inflight, 0);
  s->events.assign(max_inflight, nullptr);
  for (int i = 0; i < max_inflight; ++i) {
    if (cudaMalloc(&s->ws[2 * i], std::max<size_t>(s->ws_blocked, 256)) != cudaSuccess ||
        cudaMalloc(&s->ws[2 * i + 1], std::max<size_t>(s->ws_spectral, 256)) != cudaSuccess ||
        cudaEventCreateWithFlags(&s->events[i], cudaEventDisableTiming) != cudaSuccess) {
      smx_serve_destroy(s);
      return smx::set_error(SMX_ERR_CUDA, "smx_serve_create: device allocation failed");
    }
  }
  *out = s;
  return SMX_OK;
}

extern "C" void smx_serve_destroy(smx_server* s) {
  if (!s) return;
  cudaStreamSynchronize(s->stream);  // launches in flight, including those of a flush that failed part-way
  for (void* p : s->ws)
    if (p) cudaFree(p);
  for (cudaEvent_t e : s->events)
    if (e) cudaEventDestroy(e);
  delete s;
}

extern "C" int smx_serve_flush(smx_server* s) {
  SMX_REQUIRE(s, "smx_serve_flush: null server");
  if (s->blocked.items.empty() && s->spectral.items.empty()) return SMX_OK;
  int rc = retire(s);
  if (rc) return rc;
  if (s->flights.size() >= size_t(s->max_inflight)) {  // wait for the oldest flush to free its workspaces
    if (cudaEventSynchronize(s->flights.front().event) != cudaSuccess)
      return smx::set_error(SMX_ERR_CUDA, "smx_serve_flush: a batch launch failed");
    if ((rc = retire(s))) return rc;
  }
  int slot = 0;
  while (s->slot_busy[slot]) ++slot;
  if (!s->blocked.items.empty())
    rc = smx_blocked_eval_batch(s->blocked.plans.data(), int(s->blocked.plans.size()), s->blocked.items.data(),
                                int(s->blocked.items.size()), s->ws[2 * slot], s->ws_blocked, s->stream);
  if (!rc && !s->spectral.items.empty())
    rc = smx_spectral_eval_batch(s->spectral.plans.data(), int(s->spectral.plans.size()), s->spectral.items.data(),
                                 int(s->spectral.items.size()), s->ws[2 * slot + 1], s->ws_spectral, s->stream);
  if (!rc && cudaEventRecord(s->events[slot], s->stream) != cudaSuccess)
    rc = smx::set_error(SMX_ERR_CUDA, "smx_serve_flush: event record failed");
  if (rc) {
    // the whole flush fails: its tickets report rc, and the queue is free for new requests
    s->failed.push_back(Failed{s->flushed_end, s->next_ticket, rc});
  } else {
    s->slot_busy[slot] = 1;
    s->flights.push_back(Flight{slot, s->next_ticket, s->events[slot]});
  }
  s->flushed_end = s->next_ticket;
  s->blocked.clear();
  s->spectral.clear();
  return rc;
}

extern "C" int64_t smx_serve_submit(smx_server* s, int kind, const void* plan_host, const double* x, int64_t P,
                                    int64_t ldx, float* y) {
  SMX_REQUIRE(s && plan_host && P >= 0 && (P == 0 || (x && y)), "smx_serve_submit: bad arguments");
  SMX_REQUIRE(kind == SMX_SERVE_BLOCKED || kind == SMX_SERVE_SPECTRAL, "smx_serve_submit: unknown plan kind");
  const int d_in = kind == SMX_SERVE_BLOCKED ? static_cast<const smx_blocked*>(plan_host)->d_in
                                             : static_cast<const smx_spectral*>(plan_host)->d_in;
  SMX_REQUIRE(ldx >= d_in, "smx_serve_submit: leading dimension below d_in");
  if (kind == SMX_SERVE_SPECTRAL)
    SMX_REQUIRE(static_cast<const smx_spectral*>(plan_host)->d_out <= 16, "smx_serve_submit: more than 16 outputs");
  // a full queue (items or distinct plans of this kind) is launched first
  const bool full = kind == SMX_SERVE_BLOCKED
                        ? (s->blocked.items.size() >= size_t(s->max_items) ||
                           (s->blocked.plans.size() >= size_t(s->max_plans) &&
                            std::find(s->blocked.keys.begin(), s->blocked.keys.end(), plan_host) ==
                                s->blocked.keys.end()))
                        : (s->spectral.items.size() >= size_t(s->max_items) ||
                           (s->spectral.plans.size() >= size_t(s->max_plans) &&
                            std::find(s->spectral.keys.begin(), s->spectral.keys.end(), plan_host) ==
                                s->spectral.keys.end()));
  if (full) {
    const int rc = smx_serve_flush(s);
    if (rc) return rc;
  }
  smx_work w{};
  w.x = x;
  w.P = P;
  w.ldx = ldx;
  w.y = y;
  if (kind == SMX_SERVE_BLOCKED) {
    w.plan = s->blocked.add_plan(static_cast<const smx_blocked*>(plan_host));
    s->blocked.items.push_back(w);
  } else {
    w.plan = s->spectral.add_plan(static_cast<const smx_spectral*>(plan_host));
    s->spectral.items.push_back(w);
  }
  return s->next_ticket++;
}

extern "C" int smx_serve_poll(smx_server* s, int64_t ticket) {
  SMX_REQUIRE(s && ticket >= 0 && ticket < s->next_ticket, "smx_serve_poll: unknown ticket");
  for (const Failed& f : s->failed)
    if (ticket >= f.begin && ticket < f.end) return f.rc;
  if (ticket < s->retired_end) return 1;
  if (ticket >= s->flushed_end) return 0;  // queued, not launched yet
  const int rc = retire(s);
  if (rc) return rc;
  return ticket < s->retired_end ? 1 : 0;
}
