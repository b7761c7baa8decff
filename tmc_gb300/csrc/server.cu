// Request server: continuous batching of extraction requests on one GPU.
//
// Clients submit requests from any thread and get a ticket.  Worker threads (one CUDA stream and
// context each) take the oldest pending requests whenever they are free, as many as the HBM budget
// and the batch limit admit, and run them as one batched extraction (tmc_batch_extract).  Several
// workers keep several batches in flight, so requests that arrive while one batch runs are
// admitted into the next as soon as a worker and enough of the budget are free, and their device
// work overlaps with the running batch.
//
// Admission is by an estimate of each request's device footprint (field copy when the field is in
// host memory, per-cell scratch, per-vertex scratch and outputs at a conservative surface density);
// a request larger than the whole budget runs alone when nothing else is admitted.
//
// The request's field must stay valid until its ticket completes.  Meshes come back through
// tmc_server_wait and are released with tmc_server_release (they belong to a worker's context).
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstdio>
#include <cstring>
#include <deque>
#include <mutex>
#include <new>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../../include/tmc_gb300.h"
#include "ctx_access.h"

namespace {

struct Ticket {
  tmc_request req{};
  int64_t est = 0;       // admitted bytes
  int64_t cells = 0;     // the request's cells (batch size cap)
  bool done = false;
  tmc_status status = TMC_OK;
  std::string err;
  tmc_mesh mesh{};
  int worker = -1;
};

struct Worker {
  tmc_ctx* ctx = nullptr;
  std::mutex lock;  // guards ctx (extraction, mesh release)
  std::thread thread;
};

// bytes per cell of device footprint at a conservative surface density (0.3 vertices per cell)
int64_t estimate_bytes(const tmc_request& r) {
  const int64_t voxels = (int64_t)r.vol.nx * r.vol.ny * r.vol.nz;
  const int64_t cells = (int64_t)(r.vol.nx - 1) * (r.vol.ny - 1) * (r.vol.nz - 1);
  int64_t b = r.vol.on_device ? 0 : 4 * voxels;
  b += 16 * cells;                      // records, offsets, tile sums
  const int64_t verts = cells * 3 / 10;
  const bool dmc = r.algo == TMC_ALGO_DMC;
  b += verts * (dmc ? 24 + 16 + 200 : 24 + 24);  // positions/normals, quads or triangles, vertex scratch
  if (r.flags & (TMC_OUT_HALFEDGES | TMC_DMC_SIMPLIFY | TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333))
    b += verts * 160;                   // halfedge build and simplification buffers
  if (r.flags & (TMC_OUT_POS_F64 | TMC_OUT_TRIANGLES)) b += verts * 24;
  return b;
}

// The argument checks of the extraction entry points, made at submission so that a malformed
// request fails alone instead of failing the batch it would join.
bool request_ok(const tmc_request& r) {
  if (r.algo != TMC_ALGO_DMC && r.algo != TMC_ALGO_TMC) return false;
  const tmc_volume& v = r.vol;
  if (!v.data || v.nx < 2 || v.ny < 2 || v.nz < 2 || v.nx > 65535 || v.ny > 65535 || v.nz > 65535) return false;
  for (int d = 0; d < 3; d++)
    if (!(v.spacing[d] > 0) || !std::isfinite(v.spacing[d]) || !std::isfinite(v.origin[d])) return false;
  if ((int64_t)(v.nx - 1) * (v.ny - 1) * (v.nz - 1) > ((int64_t)1 << 32)) return false;
  if (!std::isfinite(r.iso)) return false;
  const uint32_t dmc_only = TMC_DMC_SIMPLIFY | TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333 | TMC_OUT_LOCAL;
  if (r.algo == TMC_ALGO_TMC && (r.flags & dmc_only)) return false;
  if (r.algo == TMC_ALGO_DMC && (r.flags & TMC_OUT_LOCAL) &&
      (r.flags & (TMC_DMC_SIMPLIFY | TMC_DMC_P3X3Y_COLOR | TMC_DMC_P3X3Y_ISOLATED | TMC_DMC_P3333)))
    return false;
  return true;
}

}  // namespace

struct tmc_server {
  int device = 0;
  int64_t budget = 0;
  int max_batch = 64;
  int64_t max_batch_cells = (int64_t)1 << 25;
  std::mutex m;
  std::condition_variable cv_work, cv_done;
  std::deque<int64_t> pending;
  std::unordered_map<int64_t, Ticket> tickets;
  int64_t next_ticket = 1;
  int64_t in_flight = 0;  // admitted bytes
  bool stop = false;
  std::vector<Worker*> workers;
  std::string err;
  // counters: submitted, completed, batches, requests in batches, peak admitted bytes
  int64_t n_submitted = 0, n_completed = 0, n_batches = 0, n_batched = 0, peak_bytes = 0, max_batch_seen = 0;

  void run(int w) {
    Worker* W = workers[(size_t)w];
    std::vector<int64_t> batch;
    std::vector<tmc_request> reqs;
    std::vector<tmc_mesh> outs;
    for (;;) {
      batch.clear();
      {
        std::unique_lock<std::mutex> lk(m);
        cv_work.wait(lk, [&] { return stop || !pending.empty(); });
        if (stop && pending.empty()) return;
        // admit the oldest requests while the budget and the batch limits allow: a batch's requests
        // complete together, so the cell cap keeps small requests from waiting for a large one
        int64_t batch_cells = 0;
        while (!pending.empty() && (int)batch.size() < max_batch) {
          Ticket& t = tickets[pending.front()];
          if (!batch.empty() && batch_cells + t.cells > max_batch_cells) break;
          if (!batch.empty() && in_flight + t.est > budget) break;
          if (batch.empty() && in_flight > 0 && in_flight + t.est > budget) break;  // wait for memory
          in_flight += t.est;
          batch_cells += t.cells;
          batch.push_back(pending.front());
          pending.pop_front();
        }
        if (batch.empty()) {
          // nothing fits yet: wait for a running batch to finish
          const int64_t finished = n_batches;
          cv_done.wait(lk, [&] { return stop || n_batches != finished || pending.empty(); });
          continue;
        }
        peak_bytes = std::max(peak_bytes, in_flight);
        reqs.resize(batch.size());
        for (size_t q = 0; q < batch.size(); q++) reqs[q] = tickets[batch[q]].req;
      }
      outs.assign(batch.size(), tmc_mesh{});
      tmc_status st;
      std::string msg;
      std::vector<tmc_status> sts(batch.size(), TMC_OK);
      std::vector<std::string> msgs(batch.size());
      {
        std::lock_guard<std::mutex> g(W->lock);
        if (batch.size() == 1) {
          // a batch of one: the single-volume entry point (fewer launches, no batch tables)
          const tmc_request& r = reqs[0];
          if (r.algo == TMC_ALGO_DMC) st = tmc_dmc_extract(W->ctx, &r.vol, r.iso, r.flags, &outs[0]);
          else if (r.flags & TMC_OUT_HALFEDGES) st = tmc_tmc_halfedge(W->ctx, &r.vol, r.iso, r.flags, &outs[0]);
          else st = tmc_tmc_sharedvertex(W->ctx, &r.vol, r.iso, r.flags, &outs[0]);
        } else {
          st = tmc_batch_extract(W->ctx, (int32_t)batch.size(), reqs.data(), outs.data());
        }
        if (st && batch.size() > 1) {
          // a failed batch (e.g. out of memory) is retried request by request
          for (size_t q = 0; q < batch.size(); q++) {
            sts[q] = tmc_batch_extract(W->ctx, 1, &reqs[q], &outs[q]);
            if (sts[q]) msgs[q] = tmc_last_error(W->ctx);
          }
        } else if (st) {
          sts[0] = st;
          msgs[0] = tmc_last_error(W->ctx);
        }
      }
      {
        std::lock_guard<std::mutex> lk(m);
        for (size_t q = 0; q < batch.size(); q++) {
          Ticket& t = tickets[batch[q]];
          in_flight -= t.est;
          t.done = true;
          t.status = sts[q];
          t.err = msgs[q];
          t.mesh = outs[q];
          t.worker = w;
        }
        n_completed += (int64_t)batch.size();
        n_batches++;
        n_batched += (int64_t)batch.size();
        max_batch_seen = std::max<int64_t>(max_batch_seen, (int64_t)batch.size());
      }
      cv_done.notify_all();
      cv_work.notify_all();
    }
  }
};

extern "C" {

tmc_status tmc_server_create(int device, const tmc_server_opts* opts, tmc_server** out) {
  if (!out) return TMC_ERR_INVALID_ARG;
  *out = nullptr;
  tmc_server* s = new (std::nothrow) tmc_server();
  if (!s) return TMC_ERR_OOM;
  s->device = device;
  const int nworkers = (opts && opts->workers > 0) ? opts->workers : 2;
  s->budget = (opts && opts->hbm_budget) ? (int64_t)opts->hbm_budget : (int64_t)120 << 30;
  s->max_batch = (opts && opts->max_batch > 0) ? opts->max_batch : 64;
  s->max_batch_cells = (opts && opts->max_batch_cells > 0) ? opts->max_batch_cells : (int64_t)1 << 25;
  for (int w = 0; w < nworkers; w++) {
    Worker* W = new (std::nothrow) Worker();
    if (!W) {
      tmc_server_destroy(s);
      return TMC_ERR_OOM;
    }
    const tmc_status st = tmc_ctx_create(device, nullptr, &W->ctx);
    if (st) {
      delete W;
      tmc_server_destroy(s);
      return st;
    }
    // one pool of pinned result blocks for all workers: a request's result block comes from any
    // earlier request's, whichever worker ran it (no first-use pinning inside a request's latency)
    if (w > 0) tmc::ctx_share_pinned(W->ctx, s->workers[0]->ctx);
    s->workers.push_back(W);
  }
  for (int w = 0; w < nworkers; w++) s->workers[(size_t)w]->thread = std::thread([s, w] { s->run(w); });
  *out = s;
  return TMC_OK;
}

tmc_status tmc_server_destroy(tmc_server* s) {
  if (!s) return TMC_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(s->m);
    s->stop = true;
  }
  s->cv_work.notify_all();
  s->cv_done.notify_all();
  for (Worker* W : s->workers)
    if (W->thread.joinable()) W->thread.join();
  // meshes never collected by their clients
  for (auto& kv : s->tickets) {
    Ticket& t = kv.second;
    if (t.done && t.worker >= 0 && t.mesh.priv) tmc_mesh_free(s->workers[(size_t)t.worker]->ctx, &t.mesh);
  }
  for (Worker* W : s->workers) {
    if (W->ctx) tmc_ctx_destroy(W->ctx);
    delete W;
  }
  delete s;
  return TMC_OK;
}

tmc_status tmc_server_submit(tmc_server* s, const tmc_request* req, int64_t* ticket) {
  if (!s || !req || !ticket) return TMC_ERR_INVALID_ARG;
  {
    std::lock_guard<std::mutex> lk(s->m);
    if (!request_ok(*req)) {
      s->err = "tmc_server_submit: invalid request (algorithm, grid, spacing, isovalue or flags)";
      return TMC_ERR_INVALID_ARG;
    }
    if (s->stop) return TMC_ERR_INVALID_ARG;
    const int64_t id = s->next_ticket++;
    Ticket& t = s->tickets[id];
    t.req = *req;
    t.est = estimate_bytes(*req);
    t.cells = (int64_t)(req->vol.nx - 1) * (req->vol.ny - 1) * (req->vol.nz - 1);
    s->pending.push_back(id);
    s->n_submitted++;
    *ticket = id;
  }
  s->cv_work.notify_one();
  return TMC_OK;
}

tmc_status tmc_server_poll(tmc_server* s, int64_t ticket, int32_t* done) {
  if (!s || !done) return TMC_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->m);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return TMC_ERR_INVALID_ARG;
  *done = it->second.done ? 1 : 0;
  return TMC_OK;
}

tmc_status tmc_server_wait(tmc_server* s, int64_t ticket, double timeout_s, tmc_mesh* out) {
  if (!s || !out) return TMC_ERR_INVALID_ARG;
  std::memset(out, 0, sizeof(*out));
  std::unique_lock<std::mutex> lk(s->m);
  auto it = s->tickets.find(ticket);
  if (it == s->tickets.end()) return TMC_ERR_INVALID_ARG;
  auto ready = [&] { return s->tickets[ticket].done; };
  if (timeout_s < 0) {
    s->cv_done.wait(lk, ready);
  } else if (!s->cv_done.wait_for(lk, std::chrono::duration<double>(timeout_s), ready)) {
    return TMC_ERR_TIMEOUT;
  }
  Ticket t = s->tickets[ticket];
  s->tickets.erase(ticket);
  if (t.status) {
    s->err = t.err;
    return t.status;
  }
  *out = t.mesh;
  // remember which worker owns the mesh: the reserved field carries it
  out->reserved = t.worker;
  return TMC_OK;
}

tmc_status tmc_server_release(tmc_server* s, tmc_mesh* mesh) {
  if (!s || !mesh) return TMC_ERR_INVALID_ARG;
  const int w = mesh->reserved;
  if (w < 0 || w >= (int)s->workers.size()) return TMC_ERR_INVALID_ARG;
  Worker* W = s->workers[(size_t)w];
  std::lock_guard<std::mutex> g(W->lock);
  return tmc_mesh_free(W->ctx, mesh);
}

const char* tmc_server_last_error(const tmc_server* s) { return s ? s->err.c_str() : "no server"; }

tmc_status tmc_server_stats(tmc_server* s, int64_t out[8]) {
  if (!s || !out) return TMC_ERR_INVALID_ARG;
  std::lock_guard<std::mutex> lk(s->m);
  out[0] = s->n_submitted;
  out[1] = s->n_completed;
  out[2] = s->n_batches;
  out[3] = s->n_batched;
  out[4] = s->peak_bytes;
  out[5] = s->max_batch_seen;
  out[6] = (int64_t)s->pending.size();
  out[7] = s->in_flight;
  return TMC_OK;
}

}  // extern "C"
