// Serving loop: a store of resident columns and a request loop with
// continuous batching (buff_server_* in buff_gpu.h; the reference has no
// serving layer).
//
// One host thread owns the GPU side.  Each pass it (1) retires every batch
// whose event has fired, turning its accumulators into results and freeing
// its outputs, then (2) admits waiting requests in arrival order while a
// batch slot is free and the output budget allows, and launches them as one
// persistent batched query kernel (buff_batch.cu) on that slot's stream.
// Requests that arrive while earlier batches run are admitted into the next
// free slot at once, so up to `max_inflight` batches overlap on the device.
// With `batched = 0` the same loop runs one query per launch through the
// single-column entry points (the baseline the batched form is compared to);
// in batched mode a batch that holds a single request takes that path too.
//
// Transient memory (query outputs, and the device copy of an encode
// request's host input) comes from one device arena of
// `output_budget_bytes`, handed out in power-of-two size classes; a request
// whose memory does not fit waits (and blocks later ones, keeping arrival
// order) until completions return memory.
//
// Encode requests (BUFF_Q_ENCODE) are admitted in the same arrival order but
// take no batch slot: a second host thread runs them one after another on
// its own stream (the encode reads its column's extremes back to the host to
// size the code, so it must not run on the loop thread), while the loop keeps
// admitting and retiring queries.  The new column's bytes are charged to
// `store_budget_bytes` before they are allocated; the column joins the store
// when its encode completes.
#include <cuda_runtime.h>
#include <stdint.h>
#include <string.h>

#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <new>
#include <thread>
#include <vector>

#include "buff_internal.h"

namespace {

uint64_t now_ns() {
  return (uint64_t)std::chrono::duration_cast<std::chrono::nanoseconds>(
             std::chrono::steady_clock::now().time_since_epoch())
      .count();
}

int ceil_log2(uint64_t v) {
  int c = 0;
  while ((1ull << c) < v) ++c;
  return c;
}

// Power-of-two size classes carved from one arena; freed blocks are reused
// by their class.  reset() returns everything (only with nothing in flight).
struct OutAlloc {
  uint8_t *base = nullptr;
  uint64_t cap = 0, bump = 0, used = 0;
  std::vector<uint64_t> free_[48];

  bool alloc(uint64_t bytes, uint64_t *off, int *cls) {
    const int c = ceil_log2(bytes < 4096 ? 4096 : bytes);
    if (c >= 48) return false;
    const uint64_t sz = 1ull << c;
    if (!free_[c].empty()) {
      *off = free_[c].back();
      free_[c].pop_back();
    } else if (bump + sz <= cap) {
      *off = bump;
      bump += sz;
    } else {
      return false;
    }
    *cls = c;
    used += sz;
    return true;
  }
  void release(uint64_t off, int cls) {
    free_[cls].push_back(off);
    used -= 1ull << cls;
  }
  void reset() {
    for (auto &f : free_) f.clear();
    bump = 0;
    used = 0;
  }
};

enum ReqKind : uint32_t { kQuery = 0, kEncode = 1, kRelease = 2 };

struct Req {
  buff_request r;
  uint64_t submit_ns;
  const buff_col *col;
  uint32_t *words;
  double *values;
  uint64_t off[2];  // encode: off[0]/cls[0] hold the staging of host input
  int cls[2];       // -1: no allocation
  int32_t status;
  uint32_t kind;
  uint64_t stage_bytes;  // encode: arena bytes for the device copy of host input
  uint32_t stage_rel;    // release message of an encode's staging
};

// Result area of one plain-mode request (pinned): count, 9 partials, max.
struct PlainRes {
  unsigned long long count;
  unsigned long long parts[9];
  unsigned long long max;
};

struct Slot {
  cudaStream_t s = nullptr;
  cudaEvent_t ev = nullptr;
  void *h_desc = nullptr, *d_desc = nullptr;
  unsigned long long *h_acc = nullptr, *dv_acc = nullptr;  // pinned; its device address
  uint32_t *h_flag = nullptr, *dv_flag = nullptr;         // batch completion (pinned)
  PlainRes *h_plain = nullptr, *d_plain = nullptr;
  std::vector<Req> reqs;
  bool busy = false;
  bool plain = false;  // this launch went through the single-column calls
  uint64_t seq = 0;
  uint32_t polls = 0;  // flag polls since the event was last asked
};

}  // namespace

struct buff_server {
  buff_server_config cfg;
  int device = 0;
  std::vector<buff_col *> store;  // guarded by mu once serving (encodes add to it)
  std::vector<bool> owned;        // columns made by encode requests
  uint64_t store_bytes = 0;       // guarded by mu
  OutAlloc out;
  std::vector<Slot> slots;
  uint64_t seq = 0;

  std::mutex mu;  // pending and done
  std::deque<Req> pending;
  std::vector<buff_completion> done;
  std::atomic<uint64_t> n_done{0};
  // requests pushed to `pending` and completions taken from `done` so far:
  // the loop and the pollers look at these before taking the mutex, which
  // callers spinning on an empty poll would otherwise hold for every pass
  std::atomic<uint64_t> n_pending_in{0}, n_polled{0};
  uint64_t n_pending_out = 0;  // loop thread only

  std::thread th;
  std::atomic<bool> running{false};
  std::atomic<bool> stop{false};
  std::atomic<int> loop_status{BUFF_OK};
  std::deque<Req> waiting;  // loop thread only
  uint64_t batches = 0, launched_reqs = 0;
  uint32_t warp_slots = 0;  // resident warps of the device (SMs x 64)
  uint64_t stages_out = 0;  // loop thread: encode stagings not yet returned

  // encoder thread: admitted encode requests, run one at a time on enc_s
  std::mutex enc_mu;
  std::condition_variable enc_cv;
  std::deque<Req> enc_queue;
  std::atomic<int> enc_inflight{0};  // handed to the encoder, not yet completed
  bool enc_stop = false;             // guarded by enc_mu
  std::thread enc_th;
  cudaStream_t enc_s = nullptr;
};

namespace {

uint64_t col_bytes(const buff_col *c) {
  return (uint64_t)(c->k - c->m) * c->stride + c->tail_alloc;
}

void free_outputs(buff_server *S, Req &q) {
  for (int i = 0; i < 2; ++i)
    if (q.cls[i] >= 0) {
      S->out.release(q.off[i], q.cls[i]);
      q.cls[i] = -1;
    }
}

uint64_t class_bytes(uint64_t b) { return 1ull << ceil_log2(b < 4096 ? 4096 : b); }

// Output bytes a request needs, rounded to its size classes.
uint64_t out_need(const Req &q) {
  const uint64_t n = q.col->n;
  uint64_t need = 0;
  if (q.r.ops & (BUFF_Q_RANGE | BUFF_Q_EQUAL)) need += class_bytes(((n + 31) / 32) * 4);
  if (q.r.ops & BUFF_Q_DECODE) need += class_bytes(8 * n);
  return need;
}

// Output allocations of one request; false when the budget is full now.
bool alloc_outputs(buff_server *S, Req &q) {
  q.cls[0] = q.cls[1] = -1;
  q.words = nullptr;
  q.values = nullptr;
  const uint32_t ops = q.r.ops;
  const uint64_t n = q.col->n;
  if (ops & (BUFF_Q_RANGE | BUFF_Q_EQUAL)) {
    const uint64_t nb = ((n + 31) / 32) * 4;
    if (!S->out.alloc(nb ? nb : 4, &q.off[0], &q.cls[0])) return false;
    q.words = reinterpret_cast<uint32_t *>(S->out.base + q.off[0]);
  }
  if (ops & BUFF_Q_DECODE) {
    if (!S->out.alloc(n ? 8 * n : 8, &q.off[1], &q.cls[1])) {
      free_outputs(S, q);
      return false;
    }
    q.values = reinterpret_cast<double *>(S->out.base + q.off[1]);
  }
  return true;
}

void finish(buff_server *S, Req &q, const buff_query_result &res, uint32_t column) {
  buff_completion c;
  memset(&c, 0, sizeof(c));
  c.tag = q.r.tag;
  c.status = q.status;
  c.column = column;
  c.result = res;
  c.result.status = q.status;
  c.submit_ns = q.submit_ns;
  c.done_ns = now_ns();
  if (q.kind == kEncode) {
    c.out_cls[0] = c.out_cls[1] = -1;  // its staging goes back to the loop on its own
  } else if (S->cfg.auto_release) {
    free_outputs(S, q);
  } else {
    c.words = q.words;
    c.values = q.values;
    c.out_off[0] = q.cls[0] >= 0 ? q.off[0] : ~0ull;
    c.out_off[1] = q.cls[1] >= 0 ? q.off[1] : ~0ull;
    c.out_cls[0] = q.cls[0];
    c.out_cls[1] = q.cls[1];
  }
  std::lock_guard<std::mutex> lk(S->mu);
  S->done.push_back(c);
  S->n_done.fetch_add(1, std::memory_order_release);
}

void retire(buff_server *S, Slot &sl) {
  for (size_t i = 0; i < sl.reqs.size(); ++i) {
    Req &q = sl.reqs[i];
    buff_query_result res;
    memset(&res, 0, sizeof(res));
    if (q.status == BUFF_OK) {
      buff_query uq;
      memset(&uq, 0, sizeof(uq));
      uq.col = q.col;
      uq.ops = q.r.ops;
      if (!sl.plain) {
        buffk::batch_result(uq, sl.h_acc + (size_t)buffk::kBatchAcc * i, &res);
      } else {
        const PlainRes &p = sl.h_plain[i];
        const buff_col *c = q.col;
        if (uq.ops & (BUFF_Q_RANGE | BUFF_Q_EQUAL)) res.count = p.count;
        if (uq.ops & BUFF_Q_SUM) {
          buff_sum_result sr;
          buff_sum_finish(c, reinterpret_cast<const uint64_t *>(p.parts), &sr);
          res.sum = sr.sum;
          res.n_partials = sr.n_partials;
          for (uint32_t j = 0; j < sr.n_partials && j < 9; ++j) res.partials[j] = sr.partials[j];
        }
        if ((uq.ops & BUFF_Q_MAX) && c->n) {
          res.max_code = p.max;
          res.max_value = (double)(int64_t)((uint64_t)c->base + p.max) / ldexp(1.0, (int)c->dlen);
        }
      }
    }
    finish(S, q, res, q.r.column);
  }
  sl.reqs.clear();
  sl.busy = false;
}

// One batch of admitted requests as one persistent launch.
int launch_batched(buff_server *S, Slot &sl) {
  const size_t dsz = buffk::batch_desc_size();
  const uint32_t nq = (uint32_t)sl.reqs.size();
  // one upload and one staging layout: the descriptors, the class lists, then
  // the work counters (16 bytes, padded to 64) and the accumulators, whose
  // zeros travel with the upload instead of a separate memset
  const size_t soff = (dsz * nq + 15) / 16 * 16;
  const size_t aoff = (soff + 4 * buffk::batch_sched_words(nq) + 63) / 64 * 64;
  const size_t abytes = sizeof(unsigned long long) * buffk::kBatchAcc * nq;
  uint8_t *h_base = static_cast<uint8_t *>(sl.h_desc);
  uint8_t *d_base = static_cast<uint8_t *>(sl.d_desc);
  unsigned int *d_counter = reinterpret_cast<unsigned int *>(d_base + aoff);
  unsigned long long *d_acc = reinterpret_cast<unsigned long long *>(d_base + aoff + 64);
  memset(h_base + aoff, 0, 64 + abytes);
  for (uint32_t i = 0; i < nq; ++i) {
    Req &q = sl.reqs[i];
    buff_query uq;
    memset(&uq, 0, sizeof(uq));
    uq.col = q.col;
    uq.ops = q.r.ops;
    uq.precision = q.r.precision;
    uq.pred = q.r.pred;
    uq.words = q.words;
    uq.values = q.values;
    void *d = static_cast<uint8_t *>(sl.h_desc) + dsz * i;
    q.status = buffk::batch_plan_query(uq, d_acc + (size_t)buffk::kBatchAcc * i, d);
    if (q.status != BUFF_OK) memset(d, 0, dsz);  // an invalid request: zero rows, no work
  }
  uint32_t *h_sched = reinterpret_cast<uint32_t *>(static_cast<uint8_t *>(sl.h_desc) + soff);
  const uint32_t *d_sched =
      reinterpret_cast<const uint32_t *>(static_cast<uint8_t *>(sl.d_desc) + soff);
  // tile per batch: small batches split each query over many warps (latency),
  // large ones use the configured tile (fewer, longer items).  About four
  // items per resident warp: with one (longer tiles) a batch of mixed
  // requests waited on its slowest warps (24 requests: 128 -> 169 us)
  uint64_t rows = 0;
  for (uint32_t i = 0; i < nq; ++i) rows += sl.reqs[i].col->n;
  const uint64_t slots = (uint64_t)S->warp_slots * 4;
  uint64_t tile = rows / (slots ? slots : 1);
  tile = (tile + 1023) / 1024 * 1024;
  if (tile < 1024) tile = 1024;
  if (tile > S->cfg.tune.tile_rows) tile = S->cfg.tune.tile_rows;
  buff_batch_tune t = S->cfg.tune;
  t.tile_rows = (uint32_t)tile;
  buffk::BatchSched sc;
  buffk::batch_schedule(sl.h_desc, nq, t.tile_rows, h_sched, &sc);
  cudaStream_t s = sl.s;
  // the batch's last launch copies the accumulators to sl.h_acc and then
  // writes the batch's sequence number into sl.h_flag (the loop polls it);
  // the event stays for errors
  buffk::BatchDone done;
  done.ticket = d_counter + 4;  // in the zeroed counter words
  done.acc = d_acc;
  done.hacc = sl.dv_acc;
  done.nacc = (uint32_t)(buffk::kBatchAcc * nq);
  done.flag = sl.dv_flag;
  done.seq = (uint32_t)sl.seq;
  cudaError_t e = cudaMemcpyAsync(sl.d_desc, sl.h_desc, aoff + 64 + abytes,
                                  cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = buffk::batch_launch(sl.d_desc, d_sched, sc, t, d_counter, s, &done);
  if (e == cudaSuccess) e = cudaEventRecord(sl.ev, s);
  return buffh::cuda_status(e);
}

// One request through the single-column entry points (one query per launch).
int launch_plain(Slot &sl) {
  Req &q = sl.reqs[0];
  const buff_col *c = q.col;
  cudaStream_t s = sl.s;
  void *sv = s;
  PlainRes *d = sl.d_plain;
  int st = BUFF_OK;
  const uint32_t ops = q.r.ops;
  if (ops & BUFF_Q_RANGE)
    st = buff_range_filter(c, q.r.pred, q.words, reinterpret_cast<uint64_t *>(&d->count), sv);
  else if (ops & BUFF_Q_EQUAL)
    st = buff_equal_filter(c, q.r.pred, q.words, reinterpret_cast<uint64_t *>(&d->count), sv);
  if (!st && (ops & BUFF_Q_SUM))
    st = buff_sum_partials_async(c, reinterpret_cast<uint64_t *>(d->parts), sv);
  if (!st && (ops & BUFF_Q_MAX)) st = buff_max_async(c, reinterpret_cast<uint64_t *>(&d->max), sv);
  if (!st && (ops & BUFF_Q_DECODE))
    st = q.r.precision ? buff_decode_at_precision(c, q.r.precision, q.values, sv)
                       : buff_decode(c, q.values, sv);
  q.status = st;
  cudaError_t e = cudaMemcpyAsync(sl.h_plain, d, sizeof(PlainRes), cudaMemcpyDeviceToHost, s);
  if (e == cudaSuccess) e = cudaEventRecord(sl.ev, s);
  return buffh::cuda_status(e);
}

// ---- encode requests ----

// Charges an encode's column bytes to the store budget (called by the encode
// once the code width is known, before the column is allocated).
struct EncCharge {
  buff_server *S;
  uint64_t charged;
};

int charge_store(void *ctx, uint64_t bytes) {
  EncCharge *ch = static_cast<EncCharge *>(ctx);
  buff_server *S = ch->S;
  std::lock_guard<std::mutex> lk(S->mu);
  const uint64_t cap = S->cfg.store_budget_bytes;
  if (cap && (bytes > cap || S->store_bytes > cap - bytes)) return BUFF_EFULL;
  S->store_bytes += bytes;
  ch->charged = bytes;
  return BUFF_OK;
}

// One encode request on the encoder thread: the host input is copied into
// its arena staging first, the column joins the store on success, and the
// staging returns to the loop as a release message.
void run_encode(buff_server *S, Req &q) {
  cudaStream_t s = S->enc_s;
  const void *src = q.r.values;
  int st = BUFF_OK;
  if (q.cls[0] >= 0) {
    void *dst = S->out.base + q.off[0];
    const cudaError_t e = cudaMemcpyAsync(dst, src, q.stage_bytes, cudaMemcpyDefault, s);
    if (e != cudaSuccess)
      st = buffh::cuda_status(e);
    else
      src = dst;
  }
  EncCharge ch{S, 0};
  buffh::EncodeAdmit adm{charge_store, &ch};
  buff_col *col = nullptr;
  if (st == BUFF_OK)
    st = buffh::encode_admitted(src, (int)q.r.is_f32, q.r.n, q.r.scale, q.r.flags, s, &adm, &col);
  if (st == BUFF_OK) {
    const cudaError_t e = cudaStreamSynchronize(s);  // the column is complete
    if (e != cudaSuccess) st = buffh::cuda_status(e);
  } else {
    cudaStreamSynchronize(s);  // the staging copy may still be reading
  }
  buff_query_result res;
  memset(&res, 0, sizeof(res));
  uint32_t id = 0xFFFFFFFFu;
  {
    std::lock_guard<std::mutex> lk(S->mu);
    if (st == BUFF_OK) {
      S->store.push_back(col);
      S->owned.push_back(true);
      id = (uint32_t)(S->store.size() - 1);
      res.count = q.r.n;
    } else {
      S->store_bytes -= ch.charged;
    }
    if (q.cls[0] >= 0) {  // the staging back to the loop (it owns the arena)
      Req rel;
      memset(&rel, 0, sizeof(rel));
      rel.kind = kRelease;
      rel.stage_rel = 1;
      rel.off[0] = q.off[0];
      rel.cls[0] = q.cls[0];
      rel.cls[1] = -1;
      S->pending.push_front(rel);
      S->n_pending_in.fetch_add(1, std::memory_order_release);
    }
  }
  if (st != BUFF_OK && col) buff_col_free(col);
  q.status = st;
  finish(S, q, res, id);
}

void encoder(buff_server *S) {
  cudaSetDevice(S->device);
  for (;;) {
    Req q;
    {
      std::unique_lock<std::mutex> lk(S->enc_mu);
      S->enc_cv.wait(lk, [&] { return !S->enc_queue.empty() || S->enc_stop; });
      if (S->enc_queue.empty()) break;
      q = S->enc_queue.front();
      S->enc_queue.pop_front();
    }
    run_encode(S, q);
    S->enc_inflight.fetch_sub(1, std::memory_order_acq_rel);
  }
}

void fail_request(buff_server *S, Req &q, int status) {
  q.status = status;
  buff_query_result res;
  memset(&res, 0, sizeof(res));
  finish(S, q, res, q.kind == kEncode ? 0xFFFFFFFFu : q.r.column);
}

// Nothing holds arena memory (no batch in flight, no encode staging out,
// no outputs held by callers): the size classes may be rebuilt from scratch.
bool arena_idle(buff_server *S) {
  for (const Slot &o : S->slots)
    if (o.busy || !o.reqs.empty()) return false;
  return S->stages_out == 0 && S->cfg.auto_release;
}

// Admits the encode request at the head of the waiting queue: its staging
// (for host input) from the arena, then the encoder thread.  False when the
// staging does not fit now (the request waits at the head).
bool admit_encode(buff_server *S, Req &q) {
  q.cls[0] = q.cls[1] = -1;
  if (q.stage_bytes) {
    if (class_bytes(q.stage_bytes) > S->out.cap) {  // larger than the whole arena
      fail_request(S, q, BUFF_EFULL);
      return true;
    }
    if (!S->out.alloc(q.stage_bytes, &q.off[0], &q.cls[0])) {
      if (!arena_idle(S)) return false;
      S->out.reset();
      if (!S->out.alloc(q.stage_bytes, &q.off[0], &q.cls[0])) return false;
    }
    S->stages_out++;
  }
  S->enc_inflight.fetch_add(1, std::memory_order_acq_rel);
  {
    std::lock_guard<std::mutex> lk(S->enc_mu);
    S->enc_queue.push_back(q);
  }
  S->enc_cv.notify_one();
  return true;
}

// Waiting requests beyond the free slots before slots take batches.
constexpr size_t kQueueForBatch = 4;
// Flag polls of a busy batched slot between two questions to its event.
constexpr uint32_t kEventEvery = 64;



void loop(buff_server *S) {
  cudaSetDevice(S->device);
  const uint32_t maxb = S->cfg.batched ? S->cfg.max_batch : 1;
  for (;;) {
    bool worked = false;
    // retire finished batches: a batched launch shows its completion in its
    // flag (the event is asked only now and then, for errors); a plain one
    // in its event
    for (Slot &sl : S->slots) {
      if (!sl.busy) continue;
      if (!sl.plain) {
        if (__atomic_load_n(sl.h_flag, __ATOMIC_ACQUIRE) == (uint32_t)sl.seq) {
          retire(S, sl);
          worked = true;
          continue;
        }
        if (++sl.polls < kEventEvery) continue;
        sl.polls = 0;
      }
      const cudaError_t q = cudaEventQuery(sl.ev);
      if (q == cudaSuccess) {
        retire(S, sl);
        worked = true;
      } else if (q != cudaErrorNotReady) {
        S->loop_status.store(buffh::cuda_status(q));
        for (Req &r : sl.reqs) r.status = BUFF_ECUDA;
        retire(S, sl);
      }
    }
    if (S->n_pending_in.load(std::memory_order_acquire) != S->n_pending_out) {
      std::lock_guard<std::mutex> lk(S->mu);
      while (!S->pending.empty()) {
        Req &q = S->pending.front();
        if (q.kind == kRelease) {
          // a completed request's outputs (buff_server_release) or an encode's staging
          free_outputs(S, q);
          if (q.stage_rel) S->stages_out--;
        } else {
          S->waiting.push_back(q);
        }
        S->pending.pop_front();
        S->n_pending_out++;
        worked = true;
      }
    }
    // admit in arrival order into free slots; until the waiting requests
    // outnumber the free slots by more than kQueueForBatch each takes a slot
    // of its own (light load: latency -- a batched launch of a handful of
    // requests costs more than the same requests one by one), beyond that
    // slots take batches (throughput)
    // encode requests at the head need no slot
    while (!S->waiting.empty() && S->waiting.front().kind == kEncode) {
      if (!admit_encode(S, S->waiting.front())) break;
      S->waiting.pop_front();
      worked = true;
    }
    uint32_t free_slots = 0;
    for (const Slot &sl : S->slots) free_slots += !sl.busy;
    const uint32_t take = S->waiting.size() > free_slots + kQueueForBatch ? maxb : 1;
    for (Slot &sl : S->slots) {
      if (sl.busy || S->waiting.empty()) continue;
      while (!S->waiting.empty() && sl.reqs.size() < take) {
        Req &q = S->waiting.front();
        if (q.kind == kEncode) {
          if (!admit_encode(S, q)) break;
          S->waiting.pop_front();
          continue;
        }
        if (out_need(q) > S->out.cap) {  // larger than the whole budget
          fail_request(S, q, BUFF_EFULL);
          S->waiting.pop_front();
          continue;
        }
        if (!alloc_outputs(S, q)) {
          // wait for completions (or the caller's releases) to return memory;
          // with nothing in flight and nothing held by callers, the size
          // classes are rebuilt from scratch
          if (!arena_idle(S)) break;
          S->out.reset();
          if (!alloc_outputs(S, q)) break;
        }
        sl.reqs.push_back(q);
        S->waiting.pop_front();
      }
      if (sl.reqs.empty()) break;
      // a batch of one request goes through the single-column calls: fewer
      // steps (no descriptor upload, class lists or accumulator download)
      // and the lower latency at light load
      sl.plain = !S->cfg.batched || sl.reqs.size() == 1;
      sl.seq = ++S->seq;
      sl.polls = 0;
      const int st = sl.plain ? launch_plain(sl) : launch_batched(S, sl);
      if (st) {
        S->loop_status.store(st);
        for (Req &r : sl.reqs) r.status = st;
        retire(S, sl);
        continue;
      }
      sl.busy = true;
      S->batches++;
      S->launched_reqs += sl.reqs.size();
      worked = true;
    }
    if (!worked) {
      bool idle = S->waiting.empty() && S->enc_inflight.load(std::memory_order_acquire) == 0;
      for (Slot &sl : S->slots) idle &= !sl.busy;
      if (idle && S->stop.load()) {
        std::lock_guard<std::mutex> lk(S->mu);
        if (S->pending.empty()) break;
      }
      std::this_thread::yield();
    }
  }
}

void stop_encoder(buff_server *S) {
  if (!S->enc_th.joinable()) return;
  {
    std::lock_guard<std::mutex> lk(S->enc_mu);
    S->enc_stop = true;
  }
  S->enc_cv.notify_all();
  S->enc_th.join();
}

void destroy_slots(buff_server *S) {
  for (Slot &sl : S->slots) {
    if (sl.ev) cudaEventDestroy(sl.ev);
    if (sl.s) cudaStreamDestroy(sl.s);
    if (sl.h_desc) cudaFreeHost(sl.h_desc);
    if (sl.h_acc) cudaFreeHost(sl.h_acc);
    if (sl.h_flag) cudaFreeHost(sl.h_flag);
    if (sl.h_plain) cudaFreeHost(sl.h_plain);
    if (sl.d_desc) cudaFree(sl.d_desc);
    if (sl.d_plain) cudaFree(sl.d_plain);
  }
  S->slots.clear();
}

}  // namespace

extern "C" {

int buff_server_create(const buff_server_config *cfg, buff_server **out) {
  if (!cfg || !out) return BUFF_EINVAL;
  *out = nullptr;
  buff_server_config c = *cfg;
  if (!c.max_inflight || c.max_inflight > 64 || !c.max_batch || c.max_batch > 65536 ||
      !c.output_budget_bytes)
    return BUFF_EINVAL;
  if (c.tune.tile_rows == 0) {
    c.tune.tile_rows = 32768;
    c.tune.blocks_per_sm = 4;
    c.tune.stage = 2;
  }
  if (c.tune.tile_rows % 1024 || c.tune.blocks_per_sm < 1 || c.tune.blocks_per_sm > 8 ||
      (c.tune.stage != 1 && c.tune.stage != 2 && c.tune.stage != 4))
    return BUFF_EINVAL;
  buff_server *S = new (std::nothrow) buff_server();
  if (!S) return BUFF_ENOMEM;
  S->cfg = c;
  cudaGetDevice(&S->device);
  int rc = BUFF_OK;
  cudaError_t e = cudaMalloc(reinterpret_cast<void **>(&S->out.base), c.output_budget_bytes);
  if (e != cudaSuccess) {
    rc = buffh::cuda_status(e);
    delete S;
    return rc;
  }
  S->out.cap = c.output_budget_bytes;
  S->warp_slots = (uint32_t)buffk::num_sms(S->device) * 64u;
  if ((e = cudaStreamCreateWithFlags(&S->enc_s, cudaStreamNonBlocking)) != cudaSuccess) {
    rc = buffh::cuda_status(e);
    cudaFree(S->out.base);
    delete S;
    return rc;
  }
  S->slots.resize(c.max_inflight);
  const uint32_t mb = c.batched ? c.max_batch : 1;
  const size_t dsz = buffk::batch_desc_size();
  for (Slot &sl : S->slots) {
    if ((e = cudaStreamCreateWithFlags(&sl.s, cudaStreamNonBlocking)) != cudaSuccess) break;
    if ((e = cudaEventCreateWithFlags(&sl.ev, cudaEventDisableTiming)) != cudaSuccess) break;
    const size_t sw = 4 * buffk::batch_sched_words(mb);
    // descriptors, class lists, work counters (64) and accumulators
    const size_t stage = ((dsz * mb + 15) / 16 * 16 + sw + 63) / 64 * 64 + 64 +
                         sizeof(unsigned long long) * buffk::kBatchAcc * mb;
    if ((e = cudaMallocHost(&sl.h_desc, stage)) != cudaSuccess) break;
    if ((e = cudaMallocHost(reinterpret_cast<void **>(&sl.h_acc),
                            8 * buffk::kBatchAcc * mb)) != cudaSuccess)
      break;
    if ((e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&sl.dv_acc), sl.h_acc, 0)) !=
        cudaSuccess)
      break;
    if ((e = cudaMallocHost(reinterpret_cast<void **>(&sl.h_flag), 64)) != cudaSuccess) break;
    *sl.h_flag = 0;
    if ((e = cudaHostGetDevicePointer(reinterpret_cast<void **>(&sl.dv_flag), sl.h_flag, 0)) !=
        cudaSuccess)
      break;
    if ((e = cudaMallocHost(reinterpret_cast<void **>(&sl.h_plain), sizeof(PlainRes))) != cudaSuccess)
      break;
    if ((e = cudaMalloc(&sl.d_desc, stage)) != cudaSuccess) break;
    if ((e = cudaMalloc(reinterpret_cast<void **>(&sl.d_plain), sizeof(PlainRes))) != cudaSuccess)
      break;
    sl.reqs.reserve(mb);
  }
  if (e != cudaSuccess) {
    rc = buffh::cuda_status(e);
    destroy_slots(S);
    cudaStreamDestroy(S->enc_s);
    cudaFree(S->out.base);
    delete S;
    return rc;
  }
  *out = S;
  return BUFF_OK;
}

int buff_server_add_column(buff_server *S, buff_col *col, uint32_t *id) {
  if (!S || !col || !id) return BUFF_EINVAL;
  if (col->layout != 0) return BUFF_ENOTSUP;
  if (S->running.load()) return BUFF_EINVAL;  // the store is fixed while serving
  const uint64_t b = col_bytes(col);
  if (S->cfg.store_budget_bytes && S->store_bytes + b > S->cfg.store_budget_bytes)
    return BUFF_EFULL;
  std::lock_guard<std::mutex> lk(S->mu);
  S->store.push_back(col);
  S->owned.push_back(false);
  S->store_bytes += b;
  *id = (uint32_t)(S->store.size() - 1);
  return BUFF_OK;
}

int buff_server_column(buff_server *S, uint32_t id, const buff_col **col) {
  if (!S || !col) return BUFF_EINVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  if (id >= S->store.size()) return BUFF_EINVAL;
  *col = S->store[id];
  return BUFF_OK;
}

int buff_server_store_stats(buff_server *S, uint64_t *store_bytes, uint32_t *columns) {
  if (!S) return BUFF_EINVAL;
  std::lock_guard<std::mutex> lk(S->mu);
  if (store_bytes) *store_bytes = S->store_bytes;
  if (columns) *columns = (uint32_t)S->store.size();
  return BUFF_OK;
}

int buff_server_start(buff_server *S) {
  if (!S || S->running.load()) return BUFF_EINVAL;
  S->stop.store(false);
  {
    std::lock_guard<std::mutex> lk(S->enc_mu);
    S->enc_stop = false;
  }
  S->running.store(true);
  S->enc_th = std::thread(encoder, S);
  S->th = std::thread(loop, S);
  return BUFF_OK;
}

int buff_server_submit(buff_server *S, const buff_request *reqs, uint32_t n) {
  if (!S || (n && !reqs)) return BUFF_EINVAL;
  const uint64_t t = now_ns();
  // where an encode's input lies (a device pointer query per encode request),
  // before taking the lock
  bool any_encode = false;
  for (uint32_t i = 0; i < n; ++i) any_encode |= (reqs[i].ops & BUFF_Q_ENCODE) != 0;
  std::vector<uint64_t> stage(any_encode ? n : 0, 0);
  for (uint32_t i = 0; any_encode && i < n; ++i) {
    const buff_request &r = reqs[i];
    if (r.ops != BUFF_Q_ENCODE || !r.values || !r.n) continue;
    const uint64_t bytes = r.n * (r.is_f32 ? 4u : 8u);
    if (!buffh::is_device_ptr(r.values) || (reinterpret_cast<uintptr_t>(r.values) & 15))
      stage[i] = bytes;
  }
  std::lock_guard<std::mutex> lk(S->mu);
  for (uint32_t i = 0; i < n; ++i) {
    Req q;
    memset(&q, 0, sizeof(q));
    q.r = reqs[i];
    q.submit_ns = t;
    q.cls[0] = q.cls[1] = -1;
    bool bad;
    if (reqs[i].ops & BUFF_Q_ENCODE) {
      q.kind = kEncode;
      q.stage_bytes = any_encode ? stage[i] : 0;
      bad = reqs[i].ops != BUFF_Q_ENCODE || (reqs[i].n && !reqs[i].values) ||
            reqs[i].n > BUFF_MAX_ROWS;
    } else {
      // the batched plan's checks, so that a request answers the same
      // whether it runs in a batch or through the single-column calls
      const uint32_t ops = reqs[i].ops;
      const uint32_t known = BUFF_Q_RANGE | BUFF_Q_EQUAL | BUFF_Q_SUM | BUFF_Q_MAX | BUFF_Q_DECODE;
      q.kind = kQuery;
      bad = reqs[i].column >= S->store.size() || !ops || (ops & ~known) ||
            ((ops & BUFF_Q_RANGE) && (ops & BUFF_Q_EQUAL));
    }
    if (bad) {
      buff_completion c;
      memset(&c, 0, sizeof(c));
      c.tag = reqs[i].tag;
      c.status = BUFF_EINVAL;
      c.column = reqs[i].column;
      c.result.status = BUFF_EINVAL;
      c.out_cls[0] = c.out_cls[1] = -1;
      c.submit_ns = c.done_ns = t;
      S->done.push_back(c);
      S->n_done.fetch_add(1, std::memory_order_release);
      continue;
    }
    if (q.kind == kQuery) q.col = S->store[reqs[i].column];
    S->pending.push_back(q);
    S->n_pending_in.fetch_add(1, std::memory_order_release);
  }
  return BUFF_OK;
}

int buff_server_poll(buff_server *S, buff_completion *out, uint32_t cap, uint32_t *n) {
  if (!S || !n || (cap && !out)) return BUFF_EINVAL;
  *n = 0;
  if (S->n_done.load(std::memory_order_acquire) == S->n_polled.load(std::memory_order_relaxed))
    return BUFF_OK;  // nothing new: no mutex
  std::lock_guard<std::mutex> lk(S->mu);
  const uint32_t m = (uint32_t)(S->done.size() < cap ? S->done.size() : cap);
  for (uint32_t i = 0; i < m; ++i) out[i] = S->done[i];
  S->done.erase(S->done.begin(), S->done.begin() + m);
  S->n_polled.fetch_add(m, std::memory_order_relaxed);
  *n = m;
  return BUFF_OK;
}

int buff_server_release(buff_server *S, const buff_completion *c) {
  if (!S || !c) return BUFF_EINVAL;
  // The loop thread owns the output allocator: the release travels to it as
  // a request without a column, taken before any waiting request.
  Req q;
  memset(&q, 0, sizeof(q));
  q.kind = kRelease;
  q.cls[0] = c->out_cls[0];
  q.cls[1] = c->out_cls[1];
  q.off[0] = c->out_off[0];
  q.off[1] = c->out_off[1];
  q.col = nullptr;
  std::lock_guard<std::mutex> lk(S->mu);
  S->pending.push_front(q);
  S->n_pending_in.fetch_add(1, std::memory_order_release);
  return BUFF_OK;
}

int buff_server_stop(buff_server *S) {
  if (!S) return BUFF_EINVAL;
  if (S->running.load()) {
    S->stop.store(true);
    if (S->th.joinable()) S->th.join();  // exits once every request has completed
    stop_encoder(S);
    S->running.store(false);
  }
  return S->loop_status.load();
}

int buff_server_free(buff_server *S) {
  if (!S) return BUFF_EINVAL;
  buff_server_stop(S);
  cudaDeviceSynchronize();
  destroy_slots(S);
  for (size_t i = 0; i < S->store.size(); ++i)
    if (S->owned[i]) buff_col_free(S->store[i]);
  if (S->enc_s) cudaStreamDestroy(S->enc_s);
  cudaFree(S->out.base);
  delete S;
  return BUFF_OK;
}

int buff_server_stats(buff_server *S, uint64_t *batches, uint64_t *requests,
                      uint64_t *output_bytes_in_use) {
  if (!S) return BUFF_EINVAL;
  if (batches) *batches = S->batches;
  if (requests) *requests = S->launched_reqs;
  if (output_bytes_in_use) *output_bytes_in_use = S->out.used;
  return BUFF_OK;
}

int buff_server_replay(buff_server *S, const buff_request *reqs, const uint64_t *arrival_ns,
                       uint32_t n, uint64_t *latency_ns, buff_query_result *results,
                       double *wall_s) {
  if (!S || (n && (!reqs || !arrival_ns || !latency_ns))) return BUFF_EINVAL;
  if (!S->running.load()) return BUFF_EINVAL;
  std::vector<uint64_t> due(n);
  const uint64_t t0 = now_ns() + 1000000;  // 1 ms to let the feeder start
  for (uint32_t i = 0; i < n; ++i) due[i] = t0 + arrival_ns[i];
  std::vector<buff_request> tagged(reqs, reqs + n);
  for (uint32_t i = 0; i < n; ++i) tagged[i].tag = i;
  std::thread feeder([&]() {
    uint32_t i = 0;
    while (i < n) {
      const uint64_t t = now_ns();
      uint32_t j = i;
      while (j < n && due[j] <= t) ++j;
      if (j > i) {
        buff_server_submit(S, tagged.data() + i, j - i);
        i = j;
      } else {
        std::this_thread::yield();
      }
    }
  });
  std::vector<buff_completion> buf(4096);
  uint32_t got = 0;
  uint64_t last = t0;
  int rc = BUFF_OK;
  while (got < n) {
    uint32_t m = 0;
    buff_server_poll(S, buf.data(), (uint32_t)buf.size(), &m);
    for (uint32_t k = 0; k < m; ++k) {
      const buff_completion &c = buf[k];
      const uint64_t i = c.tag;
      if (i >= n) continue;
      latency_ns[i] = c.done_ns > due[i] ? c.done_ns - due[i] : 0;
      if (results) results[i] = c.result;
      if (c.status && !rc) rc = c.status;
      if (c.done_ns > last) last = c.done_ns;
      if (!S->cfg.auto_release) buff_server_release(S, &c);
      ++got;
    }
    if (!m) std::this_thread::yield();
    const int ls = S->loop_status.load();
    if (ls != BUFF_OK) {
      rc = ls;
      break;
    }
  }
  feeder.join();
  if (wall_s) *wall_s = (double)(last - t0) / 1e9;
  return rc;
}

}  // extern "C"
