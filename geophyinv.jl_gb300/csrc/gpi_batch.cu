// gpi_batch.cu -- several forward plans advanced together (gpi_batch_*).
//
// A batch holds 2-D forward plans of one physics, each prepared as for
// gpi_run (medium, CPML profiles, sources, receivers) and each at its own
// time step.  Every time step of the batch issues the aux work of every
// member (each at its own step index: source amounts, records; one launch
// in the replayed runs, one per member for single steps) and then ONE
// launch per tile class of the step kernel over the tiles of every member: a tile
// carries its member's slot in the high half of its shot field, and the
// block reads that member's arguments (grid, buffers, coefficients, CPML
// strips, injection cells) from a device table built when the membership
// changes.  Members stepping together flip their ping-pong buffers
// together, so the table holds each member's arguments for both buffer
// parities.  Runs of 16 steps are captured once per membership as a CUDA
// graph and replayed.  A member that reaches its last step runs its tail
// (the velocity records of the last step and the extra velocity half step)
// and leaves; its records can then be read as after gpi_run.  The arithmetic
// of every cell is the one of a single plan's run, so a member's results
// equal its own gpi_run's bit for bit.
//
// No counterpart in the reference: update!(pa) runs one experiment at a
// time on each Distributed worker (src/fdtd/propagate.jl:100-106).
#include <algorithm>
#include <vector>

#include "gpi_internal.cuh"

using gpi::Plan;

namespace {

constexpr int kChunk = 16;  // steps per captured graph (even: buffers return to their parity)

struct Member {
  gpi_plan *plan = nullptr;
  int step = 0;                  // steps issued
  cudaStream_t home = nullptr;   // the plan's stream before it joined
};

}  // namespace

struct gpi_batch {
  int device = 0;
  int physics = -1;  // of the members (-1: none yet)
  cudaStream_t st = nullptr, own = nullptr;
  cudaStream_t side[3] = {};
  cudaEvent_t ev_fork = nullptr, ev_join[3] = {};
  std::vector<Member> mem;
  std::vector<gpi_plan *> finished;
  // launch tables of the current members
  bool dirty = true;
  void *d_args = nullptr;
  int4 *d_tiles = nullptr;
  void *d_aux = nullptr;  // members' aux arguments [member][parity]
  int *d_aux_first = nullptr;  // first aux block of each member (+ the total)
  int aux_blocks = 0;
  int n[4] = {}, first[4] = {};
  size_t smem[4] = {};
  int par = 0;  // buffer parity since the tables were built
  cudaGraphExec_t chunk = nullptr;
  int64_t launches = 0;
  std::string err;
};

namespace {

thread_local std::string g_batch_err;

int bfail(gpi_batch *b, int code, const std::string &msg) {
  if (b)
    b->err = msg;
  else
    g_batch_err = msg;
  return code;
}
#define B_CUDA(b, call)                                                                        \
  do {                                                                                         \
    cudaError_t e_ = (call);                                                                   \
    if (e_ != cudaSuccess) return bfail((b), GPI_E_CUDA, std::string(#call) + ": " + cudaGetErrorString(e_)); \
  } while (0)

void free_tables(gpi_batch *b) {
  if (b->chunk) cudaGraphExecDestroy(b->chunk);
  b->chunk = nullptr;
  if (b->d_args) cudaFreeAsync(b->d_args, b->st);
  if (b->d_tiles) cudaFreeAsync(b->d_tiles, b->st);
  if (b->d_aux) cudaFreeAsync(b->d_aux, b->st);
  if (b->d_aux_first) cudaFreeAsync(b->d_aux_first, b->st);
  b->d_args = nullptr;
  b->d_tiles = nullptr;
  b->d_aux = nullptr;
  b->d_aux_first = nullptr;
}

// the argument table ([member][class][parity]) and the tagged tiles of every
// class, from the members' current buffers
int build_tables(gpi_batch *b) {
  free_tables(b);
  const bool ac = b->physics == GPI_ACOUSTIC;
  const size_t ab = ac ? gpi::a2_args_bytes() : gpi::e2_args_bytes();
  const int nm = (int)b->mem.size();
  std::vector<unsigned char> args((size_t)nm * 8 * ab);
  const size_t xb = gpi::aux_args_bytes();
  std::vector<unsigned char> aux((size_t)nm * 2 * xb);
  std::vector<int> aux_first(nm + 1, 0);
  std::vector<int4> tiles[4];
  for (int m = 0; m < 4; m++) b->smem[m] = 0;
  for (int k = 0; k < nm; k++) {
    Plan &p = b->mem[k].plan->p;
    aux_first[k + 1] = aux_first[k] + gpi::aux_batch_args(&p, aux.data() + (size_t)k * 2 * xb);
    size_t sm[4];
    if (ac)
      gpi::a2_batch_args(&p, args.data() + (size_t)k * 8 * ab, sm);
    else
      gpi::e2_batch_args(&p, args.data() + (size_t)k * 8 * ab, sm);
    int at = 0;
    for (int m = 0; m < 4; m++) {
      b->smem[m] = std::max(b->smem[m], sm[m]);
      for (int i = 0; i < p.n_tiles[m]; i++, at++) {
        int4 t = p.h_tiles[at];
        t.w = (t.w & 0xffff) | (k << 16);
        tiles[m].push_back(t);
      }
    }
  }
  std::vector<int4> all;
  for (int m = 0; m < 4; m++) {
    b->first[m] = (int)all.size();
    b->n[m] = (int)tiles[m].size();
    all.insert(all.end(), tiles[m].begin(), tiles[m].end());
  }
  if (!all.empty()) {
    B_CUDA(b, gpi::pool_alloc(&b->d_args, args.size(), b->st));
    B_CUDA(b, gpi::pool_alloc((void **)&b->d_tiles, all.size() * sizeof(int4), b->st));
    B_CUDA(b, cudaMemcpyAsync(b->d_args, args.data(), args.size(), cudaMemcpyHostToDevice, b->st));
    B_CUDA(b, cudaMemcpyAsync(b->d_tiles, all.data(), all.size() * sizeof(int4), cudaMemcpyHostToDevice, b->st));
  }
  b->aux_blocks = aux_first[nm];
  if (nm > 0) {
    B_CUDA(b, gpi::pool_alloc(&b->d_aux, aux.size(), b->st));
    B_CUDA(b, gpi::pool_alloc((void **)&b->d_aux_first, aux_first.size() * sizeof(int), b->st));
    B_CUDA(b, cudaMemcpyAsync(b->d_aux, aux.data(), aux.size(), cudaMemcpyHostToDevice, b->st));
    B_CUDA(b, cudaMemcpyAsync(b->d_aux_first, aux_first.data(), aux_first.size() * sizeof(int), cudaMemcpyHostToDevice,
                              b->st));
  }
  // (the host arrays are pageable: the copies are done when these return)
  b->par = 0;
  b->dirty = false;
  return GPI_OK;
}

// one launch per tile class over the tiles of every member, the long
// classes first on side streams (as a single plan's step)
int launch_classes(gpi_batch *b) {
  const bool ac = b->physics == GPI_ACOUSTIC;
  Plan &p0 = b->mem[0].plan->p;
  const int groups = (b->n[0] > 0) + (b->n[1] > 0) + (b->n[2] > 0) + (b->n[3] > 0);
  const bool fork = groups > 1 && b->side[0];
  cudaStream_t st[3] = {b->st, b->st, b->st};
  if (fork) {
    B_CUDA(b, cudaEventRecord(b->ev_fork, b->st));
    for (int k = 0; k < 3; k++) {
      B_CUDA(b, cudaStreamWaitEvent(b->side[k], b->ev_fork, 0));
      st[k] = b->side[k];
    }
  }
  const int order[4] = {3, 2, 1, 0};
  const cudaStream_t on[4] = {st[0], st[1], st[2], b->st};
  for (int i = 0; i < 4; i++) {
    const int m = order[i];
    if (b->n[m] == 0) continue;
    const int4 *t = b->d_tiles + b->first[m];
    int rc = ac ? gpi::a2_batch_launch(&p0, m, b->d_args, t, b->n[m], b->par, b->smem[m], on[i])
                : gpi::e2_batch_launch(&p0, m, b->d_args, t, b->n[m], b->par, b->smem[m], on[i]);
    if (rc) return bfail(b, rc, p0.err);
    b->launches++;
  }
  if (fork)
    for (int k = 0; k < 3; k++) {
      B_CUDA(b, cudaEventRecord(b->ev_join[k], b->side[k]));
      B_CUDA(b, cudaStreamWaitEvent(b->st, b->ev_join[k], 0));
    }
  return GPI_OK;
}

// one plain step of every member
int plain_step(gpi_batch *b) {
  for (auto &m : b->mem) {
    Plan &p = m.plan->p;
    if (int rc = gpi::aux_step(&p, m.step + 1, GPI_FORWARD)) return bfail(b, rc, p.err);
    b->launches++;
  }
  if (int rc = launch_classes(b)) return rc;
  for (auto &m : b->mem) {
    m.plan->p.cur[0] ^= 1;
    m.step++;
  }
  b->par ^= 1;
  return GPI_OK;
}

// kChunk steps of every member as one graph (captured at parity 0 with the
// members' step counters on the device), replayed
int chunk_steps(gpi_batch *b) {
  if (!b->chunk) {
    // kernel attributes are set outside the capture
    Plan &p0 = b->mem[0].plan->p;
    for (int m = 0; m < 4; m++) {
      const int rc = b->physics == GPI_ACOUSTIC
                         ? gpi::a2_batch_launch(&p0, m, b->d_args, nullptr, 0, 0, b->smem[m], b->st)
                         : gpi::e2_batch_launch(&p0, m, b->d_args, nullptr, 0, 0, b->smem[m], b->st);
      if (rc) return bfail(b, rc, p0.err);
    }
    const int par0 = b->par;
    std::vector<int> cur0;
    for (auto &m : b->mem) cur0.push_back(m.plan->p.cur[0]);
    B_CUDA(b, cudaStreamBeginCapture(b->st, cudaStreamCaptureModeThreadLocal));
    int rc = GPI_OK;
    for (int k = 0; k < kChunk && !rc; k++) {
      // every member's records and source amounts in one launch
      if ((rc = gpi::aux_batch_launch(&p0, b->d_aux, b->d_aux_first, (int)b->mem.size(), b->aux_blocks, b->par, k,
                                      b->st)))
        rc = bfail(b, rc, p0.err);
      else
        b->launches++;
      if (!rc) rc = launch_classes(b);
      for (auto &m : b->mem) m.plan->p.cur[0] ^= 1;
      b->par ^= 1;
    }
    for (auto &m : b->mem)
      if (!rc && (rc = gpi::set_step(&m.plan->p, kChunk, 1))) rc = bfail(b, rc, m.plan->p.err);
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(b->st, &graph);
    if (!rc && e != cudaSuccess) rc = bfail(b, GPI_E_CUDA, std::string("graph capture: ") + cudaGetErrorString(e));
    if (!rc && cudaGraphInstantiate(&b->chunk, graph, 0) != cudaSuccess) {
      b->chunk = nullptr;
      rc = bfail(b, GPI_E_CUDA, "graph instantiation failed");
    }
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    // a whole chunk returns every buffer to its parity; the replay below
    // does the steps
    b->par = par0;
    for (size_t k = 0; k < b->mem.size(); k++) b->mem[k].plan->p.cur[0] = cur0[k];
    if (rc) return rc;
  }
  B_CUDA(b, cudaGraphLaunch(b->chunk, b->st));
  for (auto &m : b->mem) m.step += kChunk;  // even: buffers and parity as before
  return GPI_OK;
}

}  // namespace

extern "C" {

int gpi_batch_create(int device, void *stream, gpi_batch **out) {
  if (!out) return bfail(nullptr, GPI_E_INVALID, "null argument");
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || device < 0 || device >= ndev) {
    cudaGetLastError();
    return bfail(nullptr, GPI_E_CUDA, "no such CUDA device");
  }
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(device);
  gpi_batch *b = new gpi_batch();
  b->device = device;
  bool ok = true;
  if (stream) {
    b->st = (cudaStream_t)stream;
  } else {
    ok = cudaStreamCreateWithFlags(&b->own, cudaStreamNonBlocking) == cudaSuccess;
    b->st = b->own;
  }
  int lo = 0, hi = 0;
  cudaDeviceGetStreamPriorityRange(&lo, &hi);
  ok = ok && cudaEventCreateWithFlags(&b->ev_fork, cudaEventDisableTiming) == cudaSuccess;
  for (int k = 0; k < 3 && ok; k++)
    ok = cudaStreamCreateWithPriority(&b->side[k], cudaStreamNonBlocking, hi) == cudaSuccess &&
         cudaEventCreateWithFlags(&b->ev_join[k], cudaEventDisableTiming) == cudaSuccess;
  cudaSetDevice(prev);
  if (!ok) {
    cudaGetLastError();
    gpi_batch_destroy(b);
    return bfail(nullptr, GPI_E_CUDA, "stream or event creation failed");
  }
  *out = b;
  return GPI_OK;
}

int gpi_batch_add(gpi_batch *b, gpi_plan *plan) {
  if (!b || !plan) return bfail(b, GPI_E_INVALID, "null argument");
  Plan &p = plan->p;
  if (p.device != b->device) return bfail(b, GPI_E_INVALID, "plan on another device");
  if (p.d.ndim != 2 || p.d.npw != 1 || p.ck_slots > 0 || p.snap_buf || p.have_born || p.illum || p.d.order != 4)
    return bfail(b, GPI_E_UNSUPPORTED,
                 "batches take 2-D forward plans of stencil order 4 (npw = 1) without snapshots or illumination");
  if (b->physics >= 0 && p.d.physics != b->physics) return bfail(b, GPI_E_INVALID, "plans of one physics per batch");
  if (b->mem.size() >= 32767) return bfail(b, GPI_E_INVALID, "batch full");
  for (auto &m : b->mem)
    if (m.plan == plan) return bfail(b, GPI_E_INVALID, "plan already in the batch");
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(b->device);
  // the plan's set-up work (on its own stream) comes before its first step
  cudaEvent_t ev = nullptr;
  int rc = GPI_OK;
  if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess ||
      cudaEventRecord(ev, p.stream) != cudaSuccess || cudaStreamWaitEvent(b->st, ev, 0) != cudaSuccess)
    rc = bfail(b, GPI_E_CUDA, "ordering the plan's set-up before the batch");
  if (ev) cudaEventDestroy(ev);
  cudaStream_t home = p.stream;
  if (!rc) {
    p.stream = b->st;
    rc = gpi::run_prepare_forward(p);
    if (rc) {
      rc = bfail(b, rc, p.err);
      p.stream = home;
    }
  }
  if (!rc) {
    b->physics = p.d.physics;
    b->mem.push_back(Member{plan, 0, home});
    b->dirty = true;
  }
  cudaGetLastError();
  cudaSetDevice(prev);
  return rc;
}

int gpi_batch_advance(gpi_batch *b, int max_steps, int *active) {
  if (!b || max_steps < 0) return bfail(b, GPI_E_INVALID, "invalid argument");
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(b->device);
  int rc = GPI_OK;
  int left = max_steps;
  while (!rc && left > 0 && !b->mem.empty()) {
    if (b->dirty && (rc = build_tables(b))) break;
    int span = left;
    for (auto &m : b->mem) span = std::min(span, m.plan->p.d.nt - m.step);
    // whole graphs while they fit, plain steps otherwise (parity 0 first);
    // a graph reads the members' step counters, set before each replay
    while (!rc && span > 0) {
      if (b->par == 0 && span >= kChunk) {
        for (auto &m : b->mem)
          if (!rc && (rc = gpi::set_step(&m.plan->p, m.step + 1, 0))) rc = bfail(b, rc, m.plan->p.err);
        if (!rc) rc = chunk_steps(b);
        span -= kChunk;
        left -= kChunk;
      } else {
        rc = plain_step(b);
        span--;
        left--;
      }
    }
    if (rc) break;
    // members at their last step: the run's tail, then out of the batch
    std::vector<Member> keep;
    for (auto &m : b->mem) {
      Plan &p = m.plan->p;
      if (m.step < p.d.nt) {
        keep.push_back(m);
        continue;
      }
      if ((rc = gpi::run_finish_forward(p))) {
        rc = bfail(b, rc, p.err);
        break;
      }
      // the plan goes back to its own stream, which waits for its work
      // only (not for the batch's later steps)
      cudaEvent_t ev = nullptr;
      if (cudaEventCreateWithFlags(&ev, cudaEventDisableTiming) != cudaSuccess || cudaEventRecord(ev, b->st) != cudaSuccess ||
          cudaStreamWaitEvent(m.home, ev, 0) != cudaSuccess) {
        rc = bfail(b, GPI_E_CUDA, "handing a finished plan over");
        if (ev) cudaEventDestroy(ev);
        break;
      }
      cudaEventDestroy(ev);
      p.stream = m.home;
      b->finished.push_back(m.plan);
    }
    if (rc) break;
    if (keep.size() != b->mem.size()) {
      b->mem.swap(keep);
      b->dirty = true;
    }
  }
  // a set of members changed by the caller (add) rebuilds at the next call
  if (active) *active = (int)b->mem.size();
  cudaSetDevice(prev);
  return rc;
}

int gpi_batch_finished(gpi_batch *b, gpi_plan **plans, int cap, int *n) {
  if (!b || !n || (cap > 0 && !plans)) return bfail(b, GPI_E_INVALID, "null argument");
  const int k = std::min(cap, (int)b->finished.size());
  for (int i = 0; i < k; i++) plans[i] = b->finished[i];
  b->finished.erase(b->finished.begin(), b->finished.begin() + k);
  *n = k;
  return GPI_OK;
}

int gpi_batch_launches(gpi_batch *b, int64_t *n) {
  if (!b || !n) return bfail(b, GPI_E_INVALID, "null argument");
  *n = b->launches;
  return GPI_OK;
}

const char *gpi_batch_error(const gpi_batch *b) { return b ? b->err.c_str() : g_batch_err.c_str(); }

void gpi_batch_destroy(gpi_batch *b) {
  if (!b) return;
  int prev = 0;
  cudaGetDevice(&prev);
  cudaSetDevice(b->device);
  if (b->st) cudaStreamSynchronize(b->st);
  free_tables(b);
  if (b->st) cudaStreamSynchronize(b->st);
  // plans still in the batch go back to their own streams
  for (auto &m : b->mem) m.plan->p.stream = m.home;
  for (int k = 0; k < 3; k++) {
    if (b->side[k]) cudaStreamDestroy(b->side[k]);
    if (b->ev_join[k]) cudaEventDestroy(b->ev_join[k]);
  }
  if (b->ev_fork) cudaEventDestroy(b->ev_fork);
  if (b->own) cudaStreamDestroy(b->own);
  cudaSetDevice(prev);
  delete b;
}

}  // extern "C"
