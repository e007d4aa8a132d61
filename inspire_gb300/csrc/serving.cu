// Native continuous-batching request loop.
//
// The reference answers one request per PirServer::ProcessResponse call on
// the caller's thread (crypto/pir/server/pir_server.cc:154-306). This loop
// serves many callers at once over one or more servers (queues), keeping
// each response identical to that call's:
//   * every queue owns a ring of request slots in pinned host memory; a
//     caller acquires a slot, writes its request into it, submits it, waits
//     for its ticket and reads the response from the same slot;
//   * one scheduler thread takes the submitted slots of a queue in ring
//     order, up to max_batch at a time, as soon as one of the queue's
//     in-flight batch workspaces is free: a batch is admitted while earlier
//     batches are still running, and batches of different queues and of
//     the same queue overlap on the device (one stream per workspace);
//   * the number of workspaces per queue comes from an HBM budget;
//   * small batches use the plain engine, larger ones the tensor engine.
// The device work goes through a Backend. The PIR backend runs the server's
// answer path; the loopback backend computes a fixed function of each
// request on the host after a set delay, so the scheduling logic can be
// exercised on machines without a GPU.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/inspire_pir.h"
#include "server_api.h"

namespace inspire {
namespace {

using Clock = std::chrono::steady_clock;

int Fail(std::string* err, int code, const std::string& msg) {
  if (err) *err = msg;
  return code;
}

// ---------------------------------------------------------------------------
// Backends.
// ---------------------------------------------------------------------------
class Backend {
 public:
  virtual ~Backend() = default;
  virtual int queues() const = 0;
  // Bytes per request: first_dim (padded), second_dim, packing_key, response.
  virtual void SlotBytes(int q, size_t b[4]) const = 0;
  virtual int WordBytes(int q) const = 0;
  virtual int Validate(int q, int64_t first_dim_len, std::string* err) = 0;
  virtual bool TensorOk(int q) const = 0;
  // The engine the queue's server picks for a batch of n (its tuned
  // crossover).
  virtual int ChooseEngine(int q, int n) const = 0;
  virtual int Workspaces(int q) const = 0;
  virtual int64_t WorkspaceBytes(int q) const = 0;
  virtual bool Pinned() const = 0;
  virtual int Launch(int q, int ws, const RequestSegment* segs, int nseg,
                     int engine, std::string* err) = 0;
  virtual int Query(int q, int ws) = 0;
  virtual int Finish(int q, int ws, int engine, std::string* err) = 0;
};

class PirBackend : public Backend {
 public:
  ~PirBackend() override {
    for (auto& v : ws_)
      for (Workspace* w : v) DeleteBatchWorkspace(w);
  }
  int Init(inspire_pir_server* const* servers, int n, int max_batch,
           int64_t hbm_budget, int max_workspaces, std::string* err) {
    const int64_t share = hbm_budget / std::max(1, n);
    for (int q = 0; q < n; ++q) {
      if (servers[q] == nullptr) return Fail(err, INSPIRE_INVALID_ARGUMENT, "server is null.");
      servers_.push_back(servers[q]);
      geo_.push_back(GetGeometry(servers[q]));
      const int64_t per = BatchWorkspaceBytes(servers[q], max_batch);
      bytes_.push_back(per);
      const int64_t fit = per > 0 ? share / per : 1;
      const int count = static_cast<int>(
          std::max<int64_t>(1, std::min<int64_t>(max_workspaces, fit)));
      ws_.emplace_back();
      for (int i = 0; i < count; ++i) {
        Workspace* w = nullptr;
        const int rc = NewBatchWorkspace(servers[q], max_batch, &w, err);
        if (rc != INSPIRE_OK) return rc;
        ws_.back().push_back(w);
      }
    }
    return INSPIRE_OK;
  }
  int queues() const override { return static_cast<int>(servers_.size()); }
  void SlotBytes(int q, size_t b[4]) const override {
    const ServerGeometry& g = geo_[q];
    const size_t w = g.word_bytes, d = g.d;
    b[0] = g.db_cols * w;
    b[1] = g.nsd * d * w;
    b[2] = g.npk * d * w;
    b[3] = 2 * g.l * d * w;
  }
  int WordBytes(int q) const override { return geo_[q].word_bytes; }
  int Validate(int q, int64_t len, std::string* err) override {
    return ValidateFirstDim(servers_[q], len, err);
  }
  bool TensorOk(int q) const override { return geo_[q].tensor; }
  int ChooseEngine(int q, int n) const override {
    return ResolveEngine(servers_[q], INSPIRE_ENGINE_AUTO, n);
  }
  int Workspaces(int q) const override { return static_cast<int>(ws_[q].size()); }
  int64_t WorkspaceBytes(int q) const override { return bytes_[q]; }
  bool Pinned() const override { return true; }
  int Launch(int q, int ws, const RequestSegment* segs, int nseg, int engine,
             std::string* err) override {
    return LaunchBatch(servers_[q], ws_[q][ws], segs, nseg, engine, err);
  }
  int Query(int q, int ws) override { return QueryBatch(ws_[q][ws]); }
  int Finish(int q, int ws, int engine, std::string* err) override {
    return FinishBatch(servers_[q], ws_[q][ws], engine, err);
  }

 private:
  std::vector<inspire_pir_server*> servers_;
  std::vector<ServerGeometry> geo_;
  std::vector<int64_t> bytes_;
  std::vector<std::vector<Workspace*>> ws_;
};

// Host-only stand-in for the device: response word k of a request is
// first_dim[0] * 7 + queue + k (u32 words), ready `delay_us` after launch.
// A request whose first word is 0xDEAD fails its batch.
class LoopbackBackend : public Backend {
 public:
  LoopbackBackend(int n, const int64_t* words, int workspaces, int delay_us)
      : delay_(delay_us) {
    for (int q = 0; q < n; ++q) {
      Queue qq;
      for (int i = 0; i < 4; ++i) qq.words[i] = words[4 * q + i];
      qq.slots.resize(workspaces);
      q_.push_back(qq);
    }
  }
  int queues() const override { return static_cast<int>(q_.size()); }
  void SlotBytes(int q, size_t b[4]) const override {
    for (int i = 0; i < 4; ++i) b[i] = q_[q].words[i] * 4;
  }
  int WordBytes(int) const override { return 4; }
  int Validate(int q, int64_t len, std::string* err) override {
    if (len < 1 || len > q_[q].words[0]) {
      return Fail(err, INSPIRE_INVALID_ARGUMENT,
                  "First dimension query size (" + std::to_string(len) +
                      ") is invalid for DB columns (" +
                      std::to_string(q_[q].words[0]) + ").");
    }
    return INSPIRE_OK;
  }
  bool TensorOk(int) const override { return true; }
  // The loopback device's crossover is fixed: batches of 5 or more.
  int ChooseEngine(int, int n) const override {
    return n >= 5 ? INSPIRE_ENGINE_TENSOR : INSPIRE_ENGINE_PLAIN;
  }
  int Workspaces(int q) const override { return static_cast<int>(q_[q].slots.size()); }
  int64_t WorkspaceBytes(int) const override { return 0; }
  bool Pinned() const override { return false; }
  int Launch(int q, int ws, const RequestSegment* segs, int nseg, int,
             std::string*) override {
    Slot& s = q_[q].slots[ws];
    s.segs.assign(segs, segs + nseg);
    s.ready = Clock::now() + std::chrono::microseconds(delay_);
    return INSPIRE_OK;
  }
  int Query(int q, int ws) override {
    return Clock::now() >= q_[q].slots[ws].ready ? 1 : 0;
  }
  int Finish(int q, int ws, int, std::string* err) override {
    const Queue& qq = q_[q];
    int rc = INSPIRE_OK;
    for (const RequestSegment& sg : qq.slots[ws].segs) {
      for (int i = 0; i < sg.count; ++i) {
        const uint32_t* fd =
            static_cast<const uint32_t*>(sg.first_dim) + i * qq.words[0];
        if (fd[0] == 0xDEADu) rc = Fail(err, INSPIRE_INVALID_ARGUMENT, "loopback: rejected request");
        uint32_t* r = static_cast<uint32_t*>(sg.responses) + i * qq.words[3];
        for (int64_t k = 0; k < qq.words[3]; ++k) {
          r[k] = fd[0] * 7u + static_cast<uint32_t>(q) + static_cast<uint32_t>(k);
        }
      }
    }
    return rc;
  }

 private:
  struct Slot {
    std::vector<RequestSegment> segs;
    Clock::time_point ready;
  };
  struct Queue {
    int64_t words[4];
    std::vector<Slot> slots;
  };
  std::vector<Queue> q_;
  int delay_;
};

// ---------------------------------------------------------------------------
// The scheduler.
// ---------------------------------------------------------------------------
enum SlotState : uint8_t { kFree, kFilling, kQueued, kInflight, kDone, kFailed };
constexpr int kSeqBits = 40;

struct Ring {
  int cap = 0;
  size_t bytes[4] = {0, 0, 0, 0};
  char* base[4] = {nullptr, nullptr, nullptr, nullptr};
  std::vector<uint8_t> state;
  std::vector<Clock::time_point> t_submit;
  std::vector<int> code;
  std::vector<std::string> msg;
  int64_t head = 0, tail = 0, next_launch = 0;
  char* at(int i, int64_t seq) const { return base[i] + (seq % cap) * bytes[i]; }
};

struct Batch {
  int64_t first;
  int n;
  int ws;
  int engine;
};

struct Queue {
  Ring ring;
  std::vector<int> free_ws;
  std::deque<Batch> inflight;
};

class Engine {
 public:
  Engine(std::unique_ptr<Backend> b, int max_batch, int plain_max_batch,
         int max_wait_us)
      : be_(std::move(b)),
        max_batch_(max_batch),
        plain_max_(plain_max_batch),
        wait_(std::chrono::microseconds(max_wait_us)) {}

  ~Engine() {
    {
      std::lock_guard<std::mutex> lk(mu_);
      stop_ = true;
    }
    cv_work_.notify_all();
    if (th_.joinable()) th_.join();
    for (Queue& q : q_)
      for (char* p : q.ring.base) FreeHost(p);
  }

  int Init(int ring_slots, std::string* err) {
    const int nq = be_->queues();
    q_.resize(nq);
    for (int q = 0; q < nq; ++q) {
      Ring& r = q_[q].ring;
      r.cap = ring_slots;
      be_->SlotBytes(q, r.bytes);
      for (int i = 0; i < 4; ++i) {
        const size_t n = std::max<size_t>(r.bytes[i], 4) * ring_slots;
        r.base[i] = AllocHost(n);
        if (r.base[i] == nullptr) {
          return Fail(err, INSPIRE_RESOURCE_EXHAUSTED, "pinned request ring allocation failed");
        }
        std::memset(r.base[i], 0, n);
      }
      r.state.assign(ring_slots, kFree);
      r.t_submit.resize(ring_slots);
      r.code.assign(ring_slots, INSPIRE_OK);
      r.msg.resize(ring_slots);
      for (int w = 0; w < be_->Workspaces(q); ++w) q_[q].free_ws.push_back(w);
    }
    th_ = std::thread([this] { Loop(); });
    return INSPIRE_OK;
  }

  int Acquire(int q, int timeout_ms, int64_t* ticket, void* ptr[4], std::string* err) {
    if (q < 0 || q >= static_cast<int>(q_.size())) {
      return Fail(err, INSPIRE_INVALID_ARGUMENT, "queue index out of range.");
    }
    std::unique_lock<std::mutex> lk(mu_);
    Ring& r = q_[q].ring;
    if (!cv_space_.wait_for(lk, std::chrono::milliseconds(timeout_ms),
                            [&] { return r.head - r.tail < r.cap || stop_; }) ||
        stop_) {
      return Fail(err, INSPIRE_RESOURCE_EXHAUSTED, "request ring full (slots not released).");
    }
    const int64_t seq = r.head++;
    r.state[seq % r.cap] = kFilling;
    *ticket = (static_cast<int64_t>(q) << kSeqBits) | seq;
    for (int i = 0; i < 4; ++i) ptr[i] = r.at(i, seq);
    return INSPIRE_OK;
  }

  int Submit(int64_t ticket, int64_t first_dim_len, std::string* err) {
    int q;
    int64_t seq;
    if (!Decode(ticket, &q, &seq, kFilling)) {
      return Fail(err, INSPIRE_INVALID_ARGUMENT, "ticket is not an acquired slot.");
    }
    Ring& r = q_[q].ring;
    int rc = be_->Validate(q, first_dim_len, err);
    if (rc == INSPIRE_OK) {
      // Zero-padded first dimension (pir_server.cc:221-227).
      const size_t w = be_->WordBytes(q);
      char* fd = r.at(0, seq);
      std::memset(fd + first_dim_len * w, 0, r.bytes[0] - first_dim_len * w);
    }
    {
      std::lock_guard<std::mutex> lk(mu_);
      const int i = static_cast<int>(seq % r.cap);
      r.t_submit[i] = Clock::now();
      if (rc == INSPIRE_OK) {
        r.state[i] = kQueued;
      } else {
        r.state[i] = kFailed;
        r.code[i] = rc;
        r.msg[i] = *err;
      }
    }
    if (rc == INSPIRE_OK) {
      cv_work_.notify_one();
    } else {
      cv_done_.notify_all();
    }
    return rc;
  }

  int Wait(int64_t ticket, int timeout_ms, std::string* err) {
    int q;
    int64_t seq;
    if (!Decode(ticket, &q, &seq, 255)) {
      return Fail(err, INSPIRE_INVALID_ARGUMENT, "unknown ticket.");
    }
    Ring& r = q_[q].ring;
    const int i = static_cast<int>(seq % r.cap);
    std::unique_lock<std::mutex> lk(mu_);
    auto finished = [&] { return r.state[i] == kDone || r.state[i] == kFailed; };
    if (r.state[i] == kFilling || r.state[i] == kFree) {
      return Fail(err, INSPIRE_FAILED_PRECONDITION, "ticket was not submitted.");
    }
    if (!cv_done_.wait_for(lk, std::chrono::milliseconds(timeout_ms), finished)) {
      return Fail(err, INSPIRE_DEADLINE_EXCEEDED, "request still in flight.");
    }
    if (r.state[i] == kFailed) return Fail(err, r.code[i], r.msg[i]);
    return INSPIRE_OK;
  }

  int Release(int64_t ticket) {
    int q;
    int64_t seq;
    if (!Decode(ticket, &q, &seq, 255)) return INSPIRE_INVALID_ARGUMENT;
    Ring& r = q_[q].ring;
    {
      std::lock_guard<std::mutex> lk(mu_);
      const int i = static_cast<int>(seq % r.cap);
      if (r.state[i] == kQueued || r.state[i] == kInflight) return INSPIRE_FAILED_PRECONDITION;
      r.state[i] = kFree;
      r.code[i] = INSPIRE_OK;
      r.msg[i].clear();
      while (r.tail < r.head && r.state[r.tail % r.cap] == kFree) ++r.tail;
    }
    cv_space_.notify_all();
    return INSPIRE_OK;
  }

  void Stats(inspire_serving_stats* s) {
    std::lock_guard<std::mutex> lk(mu_);
    std::memset(s, 0, sizeof(*s));
    s->requests = static_cast<int64_t>(lat_ms_.size());
    s->failed = failed_;
    s->batches = batches_;
    s->tensor_batches = tensor_batches_;
    s->mean_batch = batches_ ? static_cast<double>(batched_) / batches_ : 0.0;
    s->max_inflight = max_inflight_;
    if (!lat_ms_.empty()) {
      std::vector<double> v = lat_ms_;
      auto pct = [&](double p) {
        const size_t k = std::min(v.size() - 1, static_cast<size_t>(p * (v.size() - 1) + 0.5));
        std::nth_element(v.begin(), v.begin() + k, v.end());
        return v[k];
      };
      s->p50_ms = pct(0.50);
      s->p99_ms = pct(0.99);
      s->max_ms = *std::max_element(v.begin(), v.end());
    }
  }

  void ResetStats() {
    std::lock_guard<std::mutex> lk(mu_);
    lat_ms_.clear();
    failed_ = batches_ = tensor_batches_ = batched_ = 0;
    max_inflight_ = 0;
  }

  int QueueInfo(int q, int32_t* workspaces, int64_t* bytes, int32_t* slots) {
    if (q < 0 || q >= static_cast<int>(q_.size())) return INSPIRE_INVALID_ARGUMENT;
    if (workspaces) *workspaces = be_->Workspaces(q);
    if (bytes) *bytes = be_->WorkspaceBytes(q);
    if (slots) *slots = q_[q].ring.cap;
    return INSPIRE_OK;
  }

 private:
  char* AllocHost(size_t n) {
    void* p = nullptr;
    if (be_->Pinned()) {
      if (cudaMallocHost(&p, n) != cudaSuccess) return nullptr;
    } else {
      p = std::malloc(n);
    }
    return static_cast<char*>(p);
  }
  void FreeHost(char* p) {
    if (p == nullptr) return;
    if (be_->Pinned()) {
      cudaFreeHost(p);
    } else {
      std::free(p);
    }
  }

  // Splits a ticket; with want != 255 the slot must be in that state.
  bool Decode(int64_t ticket, int* q, int64_t* seq, int want) {
    *q = static_cast<int>(ticket >> kSeqBits);
    *seq = ticket & ((int64_t{1} << kSeqBits) - 1);
    if (ticket < 0 || *q >= static_cast<int>(q_.size())) return false;
    std::lock_guard<std::mutex> lk(mu_);
    const Ring& r = q_[*q].ring;
    if (*seq < r.tail || *seq >= r.head) return false;
    return want == 255 || r.state[*seq % r.cap] == want;
  }

  // Marks the slots of a finished (or failed) batch and records latencies.
  void Complete(Queue& qq, const Batch& b, int rc, const std::string& msg) {
    const auto now = Clock::now();
    Ring& r = qq.ring;
    for (int k = 0; k < b.n; ++k) {
      const int i = static_cast<int>((b.first + k) % r.cap);
      if (rc == INSPIRE_OK) {
        r.state[i] = kDone;
        lat_ms_.push_back(
            std::chrono::duration<double, std::milli>(now - r.t_submit[i]).count());
      } else {
        r.state[i] = kFailed;
        r.code[i] = rc;
        r.msg[i] = msg;
        ++failed_;
      }
    }
  }

  // A queue's batch is ready when it is full, when the batching window is
  // off, or when its oldest request has waited the window out.
  bool Ready(const Ring& r, int n, Clock::time_point now,
             Clock::time_point* due) const {
    if (n >= max_batch_ || wait_.count() == 0 || stop_) return true;
    const Clock::time_point d = r.t_submit[r.next_launch % r.cap] + wait_;
    if (now >= d) return true;
    *due = std::min(*due, d);
    return false;
  }

  int Queued(const Ring& r) const {
    int n = 0;
    while (n < max_batch_ && r.next_launch + n < r.head &&
           r.state[(r.next_launch + n) % r.cap] == kQueued) {
      ++n;
    }
    return n;
  }

  void Loop() {
    for (;;) {
      bool progressed = false;
      Clock::time_point due = Clock::time_point::max();
      // Retire finished batches, oldest first per queue.
      for (int q = 0; q < static_cast<int>(q_.size()); ++q) {
        Queue& qq = q_[q];
        for (;;) {
          Batch b;
          {
            std::lock_guard<std::mutex> lk(mu_);
            if (qq.inflight.empty()) break;
            b = qq.inflight.front();
          }
          const int done = be_->Query(q, b.ws);
          if (done == 0) break;
          std::string msg;
          const int rc = done < 0 ? Fail(&msg, INSPIRE_INTERNAL, "CUDA error in a batch")
                                  : be_->Finish(q, b.ws, b.engine, &msg);
          {
            std::lock_guard<std::mutex> lk(mu_);
            Complete(qq, b, rc, msg);
            qq.inflight.pop_front();
            qq.free_ws.push_back(b.ws);
          }
          cv_done_.notify_all();
          progressed = true;
        }
      }
      // Admit submitted slots into free workspaces.
      for (int q = 0; q < static_cast<int>(q_.size()); ++q) {
        Queue& qq = q_[q];
        for (;;) {
          Batch b{};
          {
            std::lock_guard<std::mutex> lk(mu_);
            Ring& r = qq.ring;
            if (qq.free_ws.empty()) break;
            const int n = Queued(r);
            // Slots that failed validation at submit are skipped over.
            if (n == 0) {
              while (r.next_launch < r.head &&
                     r.state[r.next_launch % r.cap] != kQueued &&
                     r.state[r.next_launch % r.cap] != kFilling) {
                ++r.next_launch;
              }
              break;
            }
            if (!Ready(r, n, Clock::now(), &due)) break;
            b.first = r.next_launch;
            b.n = n;
            b.ws = qq.free_ws.back();
            qq.free_ws.pop_back();
            for (int k = 0; k < n; ++k) r.state[(b.first + k) % r.cap] = kInflight;
            r.next_launch += n;
          }
          // plain_max < 0: each server's tuned crossover decides.
          if (plain_max_ < 0) {
            b.engine = be_->ChooseEngine(q, b.n);
          } else {
            b.engine = (b.n > plain_max_ && be_->TensorOk(q)) ? INSPIRE_ENGINE_TENSOR
                                                              : INSPIRE_ENGINE_PLAIN;
          }
          // At most two contiguous runs of slots (the ring wraps once).
          Ring& r = qq.ring;
          RequestSegment segs[2];
          int nseg = 0;
          int64_t seq = b.first;
          int left = b.n;
          while (left > 0) {
            const int run = static_cast<int>(
                std::min<int64_t>(left, r.cap - seq % r.cap));
            segs[nseg++] = RequestSegment{run, r.at(0, seq), r.at(1, seq),
                                          r.at(2, seq), r.at(3, seq)};
            seq += run;
            left -= run;
          }
          std::string msg;
          const int rc = be_->Launch(q, b.ws, segs, nseg, b.engine, &msg);
          {
            std::lock_guard<std::mutex> lk(mu_);
            if (rc != INSPIRE_OK) {
              Complete(qq, b, rc, msg);
              qq.free_ws.push_back(b.ws);
            } else {
              qq.inflight.push_back(b);
              ++batches_;
              batched_ += b.n;
              if (b.engine == INSPIRE_ENGINE_TENSOR) ++tensor_batches_;
              int inflight = 0;
              for (const Queue& x : q_) inflight += static_cast<int>(x.inflight.size());
              max_inflight_ = std::max(max_inflight_, inflight);
            }
          }
          if (rc != INSPIRE_OK) cv_done_.notify_all();
          progressed = true;
        }
      }
      if (!progressed) {
        std::unique_lock<std::mutex> lk(mu_);
        bool busy = false, pending = false;
        const Clock::time_point now = Clock::now();
        for (const Queue& qq : q_) {
          busy = busy || !qq.inflight.empty();
          const Ring& r = qq.ring;
          const int n = Queued(r);
          pending = pending || (n > 0 && !qq.free_ws.empty() && Ready(r, n, now, &due));
        }
        if (stop_ && !busy) return;
        if (pending) continue;
        // Poll the device while batches run, wake for the next batching
        // window to close, sleep until a submit otherwise.
        Clock::duration wait = busy ? Clock::duration(std::chrono::microseconds(50))
                                    : Clock::duration(std::chrono::milliseconds(20));
        if (due != Clock::time_point::max()) wait = std::min(wait, due - now);
        if (wait > Clock::duration::zero()) cv_work_.wait_for(lk, wait);
      }
    }
  }

  std::unique_ptr<Backend> be_;
  int max_batch_, plain_max_;
  Clock::duration wait_;
  std::vector<Queue> q_;
  std::mutex mu_;
  std::condition_variable cv_work_, cv_done_, cv_space_;
  std::thread th_;
  bool stop_ = false;
  std::vector<double> lat_ms_;
  int64_t failed_ = 0, batches_ = 0, tensor_batches_ = 0, batched_ = 0;
  int max_inflight_ = 0;
};

}  // namespace
}  // namespace inspire

struct inspire_serving {
  std::unique_ptr<inspire::Engine> engine;
};

namespace {

int Report(int code, const std::string& msg, char* err, size_t err_len) {
  if (err != nullptr && err_len > 0) {
    std::snprintf(err, err_len, "%s", code == INSPIRE_OK ? "" : msg.c_str());
  }
  return code;
}

int Start(std::unique_ptr<inspire::Backend> be, int32_t max_batch,
          int32_t plain_max_batch, int32_t max_wait_us, int32_t ring_slots,
          inspire_serving** out, char* err, size_t err_len) {
  std::string msg;
  std::unique_ptr<inspire_serving> s(new inspire_serving());
  s->engine.reset(new inspire::Engine(std::move(be), max_batch, plain_max_batch,
                                      max_wait_us));
  const int rc = s->engine->Init(ring_slots, &msg);
  if (rc != INSPIRE_OK) return Report(rc, msg, err, err_len);
  *out = s.release();
  return INSPIRE_OK;
}

}  // namespace

extern "C" {

int inspire_serving_create(inspire_pir_server* const* servers, int32_t n_servers,
                           int32_t max_batch, int32_t plain_max_batch,
                           int32_t max_wait_us, int32_t ring_slots,
                           int64_t hbm_budget, int32_t max_workspaces,
                           inspire_serving** out, char* err, size_t err_len) {
  if (out == nullptr || servers == nullptr || n_servers <= 0 || max_batch <= 0 ||
      ring_slots < max_batch || max_workspaces <= 0 || max_wait_us < 0) {
    return Report(INSPIRE_INVALID_ARGUMENT,
                  "servers/out must be set, max_batch > 0, ring_slots >= "
                  "max_batch and max_workspaces > 0.",
                  err, err_len);
  }
  *out = nullptr;
  std::string msg;
  std::unique_ptr<inspire::PirBackend> be(new inspire::PirBackend());
  const int rc = be->Init(servers, n_servers, max_batch, hbm_budget, max_workspaces, &msg);
  if (rc != INSPIRE_OK) return Report(rc, msg, err, err_len);
  return Start(std::move(be), max_batch, plain_max_batch, max_wait_us, ring_slots, out,
               err, err_len);
}

int inspire_serving_create_loopback(int32_t n_queues, const int64_t* slot_words,
                                    int32_t workspaces, int32_t delay_us,
                                    int32_t max_batch, int32_t plain_max_batch,
                                    int32_t max_wait_us, int32_t ring_slots,
                                    inspire_serving** out, char* err,
                                    size_t err_len) {
  if (out == nullptr || slot_words == nullptr || n_queues <= 0 || workspaces <= 0 ||
      max_batch <= 0 || ring_slots < max_batch || delay_us < 0 || max_wait_us < 0) {
    return Report(INSPIRE_INVALID_ARGUMENT, "invalid loopback configuration.", err,
                  err_len);
  }
  *out = nullptr;
  std::unique_ptr<inspire::Backend> be(
      new inspire::LoopbackBackend(n_queues, slot_words, workspaces, delay_us));
  return Start(std::move(be), max_batch, plain_max_batch, max_wait_us, ring_slots, out,
               err, err_len);
}

void inspire_serving_destroy(inspire_serving* s) { delete s; }

int inspire_serving_acquire(inspire_serving* s, int32_t queue, int32_t timeout_ms,
                            int64_t* ticket, void** first_dim, void** second_dim,
                            void** packing_key, void** response, char* err,
                            size_t err_len) {
  if (s == nullptr || ticket == nullptr) {
    return Report(INSPIRE_INVALID_ARGUMENT, "engine and ticket must be set.", err, err_len);
  }
  void* p[4];
  std::string msg;
  const int rc = s->engine->Acquire(queue, timeout_ms, ticket, p, &msg);
  if (rc == INSPIRE_OK) {
    if (first_dim) *first_dim = p[0];
    if (second_dim) *second_dim = p[1];
    if (packing_key) *packing_key = p[2];
    if (response) *response = p[3];
  }
  return Report(rc, msg, err, err_len);
}

int inspire_serving_submit(inspire_serving* s, int64_t ticket, int64_t first_dim_len,
                           char* err, size_t err_len) {
  if (s == nullptr) return Report(INSPIRE_INVALID_ARGUMENT, "engine is null.", err, err_len);
  std::string msg;
  const int rc = s->engine->Submit(ticket, first_dim_len, &msg);
  return Report(rc, msg, err, err_len);
}

int inspire_serving_wait(inspire_serving* s, int64_t ticket, int32_t timeout_ms,
                         char* err, size_t err_len) {
  if (s == nullptr) return Report(INSPIRE_INVALID_ARGUMENT, "engine is null.", err, err_len);
  std::string msg;
  const int rc = s->engine->Wait(ticket, timeout_ms, &msg);
  return Report(rc, msg, err, err_len);
}

int inspire_serving_release(inspire_serving* s, int64_t ticket) {
  if (s == nullptr) return INSPIRE_INVALID_ARGUMENT;
  return s->engine->Release(ticket);
}

int inspire_serving_get_stats(inspire_serving* s, inspire_serving_stats* out) {
  if (s == nullptr || out == nullptr) return INSPIRE_INVALID_ARGUMENT;
  s->engine->Stats(out);
  return INSPIRE_OK;
}

int inspire_serving_reset_stats(inspire_serving* s) {
  if (s == nullptr) return INSPIRE_INVALID_ARGUMENT;
  s->engine->ResetStats();
  return INSPIRE_OK;
}

int inspire_serving_queue_info(inspire_serving* s, int32_t queue,
                               int32_t* workspaces, int64_t* workspace_bytes,
                               int32_t* ring_slots) {
  if (s == nullptr) return INSPIRE_INVALID_ARGUMENT;
  return s->engine->QueueInfo(queue, workspaces, workspace_bytes, ring_slots);
}

}  // extern "C"
