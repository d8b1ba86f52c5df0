// gpi_server.cu -- the serving loop behind the C ABI (gpi_server_*).
//
// Requests (forward runs or gradient! evaluations of 2-D / 3-D plans of any
// size, step count and shot count) are queued in arrival order.  Each of
// max_inflight worker threads owns a CUDA stream; a free worker admits the
// request at the head of the queue as soon as the device bytes of the
// requests already admitted plus its own stay within the HBM budget (a
// request larger than the budget runs alone), builds its plan (stream-
// ordered allocation, medium, CPML profiles, sources, receivers), runs it
// with all of its shots batched into each launch and its forward runs
// replayed as captured step chunks, copies the results to the host and
// frees the plan.  Requests on different workers overlap on the GPU, and the
// host set-up of one overlaps the device work of the others.  The device
// arithmetic of a request does not depend on what else runs, so a result
// is the same alone and in a mix.
//
// A gradient request is gradient!(g, m, L2DistLoss(), dobs, pa)
// (src/fdtd/func_grad.jl:11-49): forward_save, adjoint sources
// deriv(L2DistLoss(), dobs, dcal) = 2 (dobs - dcal) reversed in time, the
// adjoint run (with the time-reversed wavefield-1 sources of
// get_source(..., Val{-1}), src/fdtd/source.jl:8-19, when the plan uses the
// boundary store), and the raw gradient accumulations summed over shots.
//
// No counterpart in the reference: its update!(pa) runs one experiment at a
// time on each Distributed worker (src/fdtd/propagate.jl:100-106).
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/gpi_fdtd.h"

namespace {

// cells per step (extended grid x shots) up to which a 2-D forward request
// joins a batch
constexpr int64_t kBatchCells = 4 << 20;

struct Proj {
  int shot = 0, field = 0, n = 0;
  std::vector<int64_t> cp, rv;
  std::vector<float> nz, data;
  bool has_data = false;
};

enum { QUEUED = 0, RUNNING = 1, DONE = 2, FAILED = 3 };

struct Job {
  int64_t id = 0;
  gpi_plan_desc desc{};
  int gradient = 0, graph = 0;
  int kind = 0;  // 0 a worker thread's; 1 + physics: the batch of 2-D forward requests of that physics
  std::vector<std::vector<float>> mod;
  std::vector<float> pml;
  std::vector<Proj> src, rec;
  size_t bytes = 0;
  int state = QUEUED;
  int status = GPI_OK;
  std::string message;
  double t_submit = 0, t_admit = 0, t_done = 0;
  std::vector<std::vector<float>> records;  // per rec entry: nt x n
  std::vector<std::vector<float>> grad;     // invK (or invlambda), rho ...: extended grid
  double loss = 0;
};

int nder_of(const gpi_plan_desc &d) {
  if (d.physics == GPI_ACOUSTIC) return d.ndim == 2 ? 4 : 6;
  return d.ndim == 2 ? 8 : 18;
}
int64_t grid_cells(const gpi_plan_desc &d) { return (int64_t)d.nz * (d.ndim == 3 ? d.ny : 1) * d.nx; }
bool is_vel(int f) { return f == GPI_VX || f == GPI_VY || f == GPI_VZ; }

}  // namespace

struct gpi_server {
  gpi_server_desc d{};
  std::mutex mu;
  std::condition_variable cv;
  std::deque<Job *> queue;
  std::map<int64_t, Job *> jobs;
  size_t used = 0;
  int inflight = 0;
  bool stop = false;
  int64_t next_id = 1;
  std::vector<std::thread> workers;
  int max_batch = 16;  // members of a batch (0: no batches)
  std::chrono::steady_clock::time_point t0 = std::chrono::steady_clock::now();
  double now() const {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  }
};

namespace {

thread_local std::string g_msg;

int sfail(int code, const std::string &m) {
  g_msg = m;
  return code;
}

// a request's plan with its medium, CPML profiles, receivers and sources,
// its set-up work on stream st
int prepare(Job &j, cudaStream_t st, gpi_plan **out) {
  gpi_plan *plan = nullptr;
  *out = nullptr;
  int rc = gpi_plan_create(&j.desc, &plan);
  auto check = [&](int r) {
    if (r && j.message.empty()) j.message = gpi_last_error(plan);
    return r;
  };
  if (rc) {
    j.message = gpi_last_error(nullptr);
    return rc;
  }
  const gpi_plan_desc &d = j.desc;
  do {
    if ((rc = check(gpi_set_stream(plan, st)))) break;
    std::vector<const float *> mp;
    for (auto &m : j.mod) mp.push_back(m.data());
    if ((rc = check(gpi_set_medium(plan, mp.data(), 0)))) break;
    const int nq = nder_of(d), P = 2 * d.npml;
    for (int q = 0; q < nq && !rc; q++) {
      const float *base = j.pml.data() + (size_t)q * 3 * P;
      rc = check(gpi_set_pml(plan, q, P, base, base + P, base + 2 * P));
    }
    if (rc) break;
    for (auto &r : j.rec)
      if ((rc = check(gpi_set_receivers(plan, r.shot, r.field, r.n, r.cp.data(), r.rv.data(), r.nz.data())))) break;
    if (rc) break;
    for (auto &s : j.src)
      if ((rc = check(gpi_set_sources(plan, 1, s.shot, s.field, s.n, s.cp.data(), s.rv.data(), s.nz.data(),
                                       s.data.data()))))
        break;
    if (rc) break;
    if (j.graph && (rc = check(gpi_set_graph(plan, j.graph)))) break;
  } while (false);
  if (rc) {
    gpi_plan_destroy(plan);
    return rc;
  }
  *out = plan;
  return GPI_OK;
}

// the records of a finished forward run
int fetch_records(Job &j, gpi_plan *plan) {
  int rc = GPI_OK;
  j.records.assign(j.rec.size(), {});
  for (size_t k = 0; k < j.rec.size() && !rc; k++) {
    j.records[k].resize((size_t)j.desc.nt * j.rec[k].n);
    rc = gpi_get_records(plan, j.rec[k].shot, j.rec[k].field, j.records[k].data(), 0);
    if (rc && j.message.empty()) j.message = gpi_last_error(plan);
  }
  return rc;
}

// the whole life of one admitted request on a worker's stream
int process(Job &j, cudaStream_t st) {
  gpi_plan *plan = nullptr;
  int rc = prepare(j, st, &plan);
  if (rc) return rc;
  auto check = [&](int r) {
    if (r && j.message.empty()) j.message = gpi_last_error(plan);
    return r;
  };
  const gpi_plan_desc &d = j.desc;
  const int nt = d.nt;
  do {
    if ((rc = check(gpi_run(plan, j.gradient ? GPI_FORWARD_SAVE : GPI_FORWARD)))) break;
    if ((rc = fetch_records(j, plan))) break;
    if (!j.gradient) break;
    // adjoint sources 2 (dobs - dcal), reversed in time, and the misfit
    // sum (dobs - dcal)^2, on the device from the records there
    double loss = 0;
    std::vector<float> zeros;
    for (size_t k = 0; k < j.rec.size() && !rc; k++) {
      const Proj &r = j.rec[k];
      if (!r.has_data) zeros.assign((size_t)nt * r.n, 0.f);
      double mis = 0;
      rc = check(gpi_set_adjoint_l2(plan, r.shot, r.field, r.has_data ? r.data.data() : zeros.data(), 0, &mis));
      loss += mis;
    }
    if (rc) break;
    j.loss = loss;
    if (d.checkpoints == 0) {
      // the boundary-store adjoint runs wavefield 1 backwards with the
      // time-reversed sources: -w shifted by one step, reversed, row 1 zero
      for (auto &s : j.src) {
        if (!is_vel(s.field)) {
          rc = sfail(GPI_E_UNSUPPORTED, "time-reversed sources act on velocities only (source.jl:8-19)");
          j.message = g_msg;
          break;
        }
        std::vector<float> w((size_t)nt * s.n, 0.f);
        for (int i = 0; i < s.n; i++)
          for (int t = 1; t < nt; t++) w[(size_t)i * nt + t] = -s.data[(size_t)i * nt + (nt - t)];
        if ((rc = check(gpi_set_sources(plan, 1, s.shot, s.field, s.n, s.cp.data(), s.rv.data(), s.nz.data(),
                                         w.data()))))
          break;
      }
      if (rc) break;
    }
    if ((rc = check(gpi_run(plan, GPI_ADJOINT)))) break;
    const int64_t n = grid_cells(d);
    j.grad.assign(2, std::vector<float>(n));
    for (int q = 0; q < 2 && !rc; q++) rc = check(gpi_get_gradient(plan, q, j.grad[q].data(), 0));
  } while (false);
  if (!rc && cudaStreamSynchronize(st) != cudaSuccess) {
    rc = GPI_E_CUDA;
    j.message = cudaGetErrorString(cudaGetLastError());
  }
  gpi_plan_destroy(plan);
  return rc;
}

// the first queued request of a kind (arrival order within each kind)
Job *first_of(gpi_server *s, int kind) {
  for (Job *j : s->queue)
    if (j->kind == kind) return j;
  return nullptr;
}

void worker(gpi_server *s) {
  cudaSetDevice(s->d.device);
  cudaStream_t st = nullptr;
  const bool have_stream = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess;
  for (;;) {
    Job *j = nullptr;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      s->cv.wait(lock, [&] {
        if (s->stop) return true;
        Job *h = first_of(s, 0);
        return h && (s->inflight == 0 || s->used + h->bytes <= s->d.hbm_budget);
      });
      if (s->stop) break;
      j = first_of(s, 0);
      s->queue.erase(std::find(s->queue.begin(), s->queue.end(), j));
      s->used += j->bytes;
      s->inflight++;
      j->state = RUNNING;
      j->t_admit = s->now();
    }
    const int rc = have_stream ? process(*j, st) : GPI_E_CUDA;
    if (!have_stream) j->message = "worker stream creation failed";
    {
      std::lock_guard<std::mutex> lock(s->mu);
      j->status = rc;
      j->state = rc ? FAILED : DONE;
      j->t_done = s->now();
      s->used -= j->bytes;
      s->inflight--;
    }
    s->cv.notify_all();
  }
  if (have_stream) cudaStreamDestroy(st);
}

// The batch of 2-D forward requests of one physics: admitted requests join
// it (their plans set up on a second stream while the batch runs), each
// gpi_batch_advance issues a stretch of steps of every member, and the
// records of the members that finished in the previous stretch are read
// while the current one runs.  At most two stretches are in flight.
void batch_worker(gpi_server *s, int physics) {
  const int kind = 1 + physics;
  constexpr int kStretch = 64;
  cudaSetDevice(s->d.device);
  cudaStream_t st = nullptr, prep = nullptr;
  cudaEvent_t ev[2] = {};
  gpi_batch *b = nullptr;
  bool ok = cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking) == cudaSuccess &&
            cudaStreamCreateWithFlags(&prep, cudaStreamNonBlocking) == cudaSuccess &&
            cudaEventCreateWithFlags(&ev[0], cudaEventDisableTiming) == cudaSuccess &&
            cudaEventCreateWithFlags(&ev[1], cudaEventDisableTiming) == cudaSuccess &&
            gpi_batch_create(s->d.device, st, &b) == GPI_OK;
  std::map<gpi_plan *, Job *> members;
  std::vector<std::pair<Job *, gpi_plan *>> finishing;  // finished in the previous stretch
  int nev = 0;
  auto complete = [&](Job *j, int rc) {
    std::lock_guard<std::mutex> lock(s->mu);
    j->status = rc;
    j->state = rc ? FAILED : DONE;
    j->t_done = s->now();
    s->used -= j->bytes;
    s->inflight--;
  };
  for (;;) {
    std::vector<Job *> admit;
    {
      std::unique_lock<std::mutex> lock(s->mu);
      if (members.empty() && finishing.empty())
        s->cv.wait(lock, [&] { return s->stop || first_of(s, kind) != nullptr; });
      if (s->stop && members.empty() && finishing.empty()) break;
      for (;;) {
        Job *h = first_of(s, kind);
        if (!h || s->stop || (int)(members.size() + admit.size()) >= s->max_batch) break;
        if (!(s->inflight == 0 || s->used + h->bytes <= s->d.hbm_budget)) break;
        s->queue.erase(std::find(s->queue.begin(), s->queue.end(), h));
        s->used += h->bytes;
        s->inflight++;
        h->state = RUNNING;
        h->t_admit = s->now();
        admit.push_back(h);
      }
    }
    for (Job *j : admit) {
      gpi_plan *plan = nullptr;
      int rc = ok ? prepare(*j, prep, &plan) : GPI_E_CUDA;
      if (!ok) j->message = "batch worker streams or batch creation failed";
      if (!rc && (rc = gpi_batch_add(b, plan))) j->message = gpi_batch_error(b);
      if (rc) {
        if (plan) gpi_plan_destroy(plan);
        complete(j, rc);
        s->cv.notify_all();
        continue;
      }
      members[plan] = j;
    }
    // at most two stretches in flight: wait for the one before the last
    if (nev >= 2) cudaEventSynchronize(ev[nev & 1]);
    int active = 0;
    int rc = ok ? gpi_batch_advance(b, kStretch, &active) : GPI_E_CUDA;
    if (ok) cudaEventRecord(ev[nev & 1], st);
    nev++;
    // records of the members that finished in the previous stretch
    for (auto &f : finishing) {
      const int r = rc ? rc : fetch_records(*f.first, f.second);
      if (rc && f.first->message.empty()) f.first->message = gpi_batch_error(b);
      gpi_plan_destroy(f.second);
      complete(f.first, r);
    }
    if (!finishing.empty()) s->cv.notify_all();
    finishing.clear();
    gpi_plan *done[64];
    int n = 0;
    do {
      if (gpi_batch_finished(b, done, 64, &n)) break;
      for (int k = 0; k < n; k++) {
        finishing.push_back({members[done[k]], done[k]});
        members.erase(done[k]);
      }
    } while (n == 64);
    if (rc) {
      // a failed stretch fails every member
      std::string msg = gpi_batch_error(b);
      for (auto &m : members) {
        m.second->message = msg;
        complete(m.second, rc);
      }
      members.clear();
      gpi_batch_destroy(b);
      b = nullptr;
      ok = gpi_batch_create(s->d.device, st, &b) == GPI_OK;
      s->cv.notify_all();
    }
  }
  if (b) gpi_batch_destroy(b);
  if (ev[0]) cudaEventDestroy(ev[0]);
  if (ev[1]) cudaEventDestroy(ev[1]);
  if (prep) cudaStreamDestroy(prep);
  if (st) cudaStreamDestroy(st);
}

Job *find(gpi_server *s, int64_t id) {
  auto it = s->jobs.find(id);
  return it == s->jobs.end() ? nullptr : it->second;
}

}  // namespace

extern "C" {

int gpi_server_create(const gpi_server_desc *desc, gpi_server **out) {
  if (!desc || !out) return sfail(GPI_E_INVALID, "null argument");
  *out = nullptr;
  if (desc->max_inflight < 1 || desc->max_inflight > 64) return sfail(GPI_E_INVALID, "max_inflight: 1..64");
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || desc->device < 0 || desc->device >= ndev) {
    cudaGetLastError();
    return sfail(GPI_E_CUDA, "no such CUDA device");
  }
  if (desc->max_batch < -1 || desc->max_batch > 4096) return sfail(GPI_E_INVALID, "max_batch: -1..4096");
  gpi_server *s = new gpi_server();
  s->d = *desc;
  s->max_batch = desc->max_batch == 0 ? 16 : desc->max_batch < 0 ? 0 : desc->max_batch;
  for (int i = 0; i < desc->max_inflight; i++) s->workers.emplace_back(worker, s);
  if (s->max_batch > 0)
    for (int ph : {GPI_ACOUSTIC, GPI_ELASTIC}) s->workers.emplace_back(batch_worker, s, ph);
  *out = s;
  return GPI_OK;
}

void gpi_server_destroy(gpi_server *s) {
  if (!s) return;
  {
    std::lock_guard<std::mutex> lock(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  // a worker finishes the request it is running before it leaves
  for (auto &t : s->workers) t.join();
  for (auto &kv : s->jobs) delete kv.second;
  delete s;
}

static int copy_proj(const gpi_proj &p, int nt, bool with_data, bool data_optional, Proj *out) {
  if (p.n < 1 || !p.colptr || !p.rowval || !p.nzval) return sfail(GPI_E_INVALID, "projection arrays");
  if (p.colptr[0] != 0) return sfail(GPI_E_INVALID, "colptr[0] must be 0");
  for (int j = 0; j < p.n; j++)
    if (p.colptr[j + 1] < p.colptr[j]) return sfail(GPI_E_INVALID, "colptr not monotone");
  const int64_t nnz = p.colptr[p.n];
  out->shot = p.shot;
  out->field = p.field;
  out->n = p.n;
  out->cp.assign(p.colptr, p.colptr + p.n + 1);
  out->rv.assign(p.rowval, p.rowval + nnz);
  out->nz.assign(p.nzval, p.nzval + nnz);
  if (with_data) {
    if (!p.data && !data_optional) return sfail(GPI_E_INVALID, "source wavelets missing");
    if (p.data) {
      out->data.assign(p.data, p.data + (size_t)nt * p.n);
      out->has_data = true;
    }
  }
  return GPI_OK;
}

int gpi_server_submit(gpi_server *s, const gpi_request *r, int64_t *id) {
  if (!s || !r || !id) return sfail(GPI_E_INVALID, "null argument");
  const gpi_plan_desc &d = r->plan;
  if (r->gradient && d.npw != 2) return sfail(GPI_E_INVALID, "a gradient request needs npw = 2");
  if (!r->gradient && d.npw != 1) return sfail(GPI_E_INVALID, "a forward request needs npw = 1");
  if (r->nsrc < 1 || r->nrec < 1 || !r->src || !r->rec || !r->mod || !r->pml)
    return sfail(GPI_E_INVALID, "sources, receivers, medium and PML profiles are required");
  size_t bytes = 0;
  if (int rc = gpi_plan_estimate(&d, &bytes)) return sfail(rc, gpi_last_error(nullptr));
  Job *j = new Job();
  j->desc = d;
  j->gradient = r->gradient;
  j->graph = r->graph;
  // small 2-D forward requests of stencil order 4 (launch-bound alone) join
  // the batch of their physics; large ones fill the device on their own
  const bool small = (int64_t)d.nz * d.nx * d.nshots <= kBatchCells;
  j->kind = (!r->gradient && d.ndim == 2 && d.order == 4 && small && s->max_batch > 0) ? 1 + d.physics : 0;
  const int nmod = d.physics == GPI_ACOUSTIC ? 2 : 3;
  const int64_t cells = grid_cells(d);
  for (int i = 0; i < nmod; i++) {
    if (!r->mod[i]) {
      delete j;
      return sfail(GPI_E_INVALID, "medium array missing");
    }
    j->mod.emplace_back(r->mod[i], r->mod[i] + cells);
  }
  j->pml.assign(r->pml, r->pml + (size_t)nder_of(d) * 3 * 2 * d.npml);
  size_t rec_floats = 0;
  for (int k = 0; k < r->nsrc; k++) {
    Proj p;
    if (int rc = copy_proj(r->src[k], d.nt, true, false, &p)) {
      delete j;
      return rc;
    }
    j->src.push_back(std::move(p));
  }
  for (int k = 0; k < r->nrec; k++) {
    Proj p;
    if (int rc = copy_proj(r->rec[k], d.nt, r->gradient != 0, true, &p)) {
      delete j;
      return rc;
    }
    rec_floats += (size_t)d.nt * p.n;
    j->rec.push_back(std::move(p));
  }
  // the plan's pool plus its record buffers (and the adjoint sources)
  j->bytes = bytes + rec_floats * sizeof(float) * (r->gradient ? 3 : 2);
  {
    std::lock_guard<std::mutex> lock(s->mu);
    j->id = s->next_id++;
    j->t_submit = s->now();
    s->jobs[j->id] = j;
    s->queue.push_back(j);
    *id = j->id;
  }
  s->cv.notify_all();
  return GPI_OK;
}

int gpi_server_poll(gpi_server *s, int64_t id, int *state) {
  if (!s || !state) return sfail(GPI_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  Job *j = find(s, id);
  if (!j) return sfail(GPI_E_INVALID, "unknown request");
  *state = j->state;
  return GPI_OK;
}

int gpi_server_wait(gpi_server *s, int64_t id) {
  if (!s) return sfail(GPI_E_INVALID, "null argument");
  std::unique_lock<std::mutex> lock(s->mu);
  Job *j = find(s, id);
  if (!j) return sfail(GPI_E_INVALID, "unknown request");
  s->cv.wait(lock, [&] { return j->state == DONE || j->state == FAILED || s->stop; });
  if (j->state == FAILED) return sfail(j->status, j->message);
  return j->state == DONE ? GPI_OK : sfail(GPI_E_STATE, "server stopped");
}

int gpi_server_records(gpi_server *s, int64_t id, int shot, int field, float *out) {
  if (!s || !out) return sfail(GPI_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  Job *j = find(s, id);
  if (!j) return sfail(GPI_E_INVALID, "unknown request");
  if (j->state != DONE) return sfail(GPI_E_STATE, "request not done");
  for (size_t k = 0; k < j->rec.size(); k++)
    if (j->rec[k].shot == shot && j->rec[k].field == field) {
      std::copy(j->records[k].begin(), j->records[k].end(), out);
      return GPI_OK;
    }
  return sfail(GPI_E_INVALID, "no such receiver entry");
}

int gpi_server_gradient(gpi_server *s, int64_t id, int param, float *out, double *loss) {
  if (!s) return sfail(GPI_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  Job *j = find(s, id);
  if (!j) return sfail(GPI_E_INVALID, "unknown request");
  if (j->state != DONE) return sfail(GPI_E_STATE, "request not done");
  if (!j->gradient) return sfail(GPI_E_INVALID, "not a gradient request");
  if (param < 0 || param >= 2) return sfail(GPI_E_INVALID, "param");
  if (out) std::copy(j->grad[param].begin(), j->grad[param].end(), out);
  if (loss) *loss = j->loss;
  return GPI_OK;
}

int gpi_server_times(gpi_server *s, int64_t id, double *t) {
  if (!s || !t) return sfail(GPI_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  Job *j = find(s, id);
  if (!j) return sfail(GPI_E_INVALID, "unknown request");
  t[0] = j->t_submit;
  t[1] = j->t_admit;
  t[2] = j->t_done;
  return GPI_OK;
}

const char *gpi_server_message(gpi_server *s, int64_t id) {
  if (!s) return g_msg.c_str();
  std::lock_guard<std::mutex> lock(s->mu);
  Job *j = find(s, id);
  return j ? j->message.c_str() : g_msg.c_str();
}

int gpi_server_release(gpi_server *s, int64_t id) {
  if (!s) return sfail(GPI_E_INVALID, "null argument");
  std::lock_guard<std::mutex> lock(s->mu);
  Job *j = find(s, id);
  if (!j) return sfail(GPI_E_INVALID, "unknown request");
  if (j->state != DONE && j->state != FAILED) return sfail(GPI_E_STATE, "request still queued or running");
  s->jobs.erase(id);
  delete j;
  return GPI_OK;
}

}  // extern "C"
