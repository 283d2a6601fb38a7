// Serving: a request loop with continuous batching over resident databases
// (the gs_server_* entry points of include/gspan_gb300.h).
//
// One server thread owns a Scheduler (its own stream, device pool and
// scratch).  Each loop iteration it applies cancellations, admits queued
// requests in arrival order while active slots and the embedding-store
// budget allow, runs one scheduler step (launch waves, finish the oldest),
// and publishes the requests that finished.  A request admitted while others
// run joins the very next wave: its DFS-tree nodes are batched with theirs.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "gs_handles.hpp"

namespace gsgb {
namespace {

using clk = std::chrono::steady_clock;

double ms_between(clk::time_point a, clk::time_point b)
{
  return std::chrono::duration<double, std::milli>(b - a).count();
}

struct Request {
  int64_t id = 0;
  int32_t db_id = 0;
  int32_t minsup = 0;
  int32_t max_edges = 0;
  int32_t state = GS_REQ_QUEUED;
  gs_status status = GS_OK;
  bool cancel = false;
  int32_t job = -1;           // scheduler job id while running
  int64_t estimate = 0;       // embedding-store bytes charged at admission
  int64_t patterns = 0;
  int64_t peak_bytes = 0;
  clk::time_point t_submit, t_admit, t_end;
  std::unique_ptr<PatternBuf> out;
};

struct HistKey {
  int32_t db, minsup, max_edges;
  bool operator<(const HistKey &o) const
  {
    if(db != o.db) return db < o.db;
    if(minsup != o.minsup) return minsup < o.minsup;
    return max_edges < o.max_edges;
  }
};

}  // namespace

class Server {
public:
  explicit Server(const gs_server_opts &o) : opt_(o)
  {
    if(opt_.max_active <= 0) opt_.max_active = 64;
    t_create_ = clk::now();
    th_ = std::thread([this] { loop(); });
  }
  ~Server()
  {
    {
      std::lock_guard<std::mutex> g(m_);
      stop_ = true;
      for(auto &kv : reqs_)
        if(kv.second->state == GS_REQ_QUEUED || kv.second->state == GS_REQ_RUNNING) kv.second->cancel = true;
    }
    cv_.notify_all();
    th_.join();
  }

  int32_t add_db(Database *db)
  {
    std::lock_guard<std::mutex> g(m_);
    dbs_.push_back(db);
    return (int32_t)dbs_.size() - 1;
  }

  gs_status submit(int32_t db_id, int32_t minsup, int32_t max_edges, int64_t *id, std::string &err)
  {
    std::lock_guard<std::mutex> g(m_);
    if(db_id < 0 || db_id >= (int32_t)dbs_.size()) {
      err = "unknown database id";
      return GS_ERR_USAGE;
    }
    if(minsup < 1) {
      err = "error: absolute_min_support < 1";
      return GS_ERR_MINSUP_TOO_SMALL;
    }
    const int32_t ng = dbs_[db_id]->host.n_graphs;
    if(minsup >= ng) {
      err = "error: user specified support " + std::to_string(minsup) + " is greater then the database size " +
            std::to_string(ng);
      return GS_ERR_MINSUP_TOO_LARGE;
    }
    std::unique_ptr<Request> r(new Request());
    r->id = next_id_++;
    r->db_id = db_id;
    r->minsup = minsup;
    r->max_edges = std::max(0, max_edges);
    r->t_submit = clk::now();
    *id = r->id;
    queue_.push_back(r->id);
    reqs_[r->id] = std::move(r);
    submitted_++;
    cv_.notify_all();
    return GS_OK;
  }

  gs_status poll(int64_t id, int32_t wait_ms, gs_request_info *info, gs_patterns **out, std::string &err)
  {
    std::unique_lock<std::mutex> l(m_);
    auto ended = [&] {
      auto it = reqs_.find(id);
      return it == reqs_.end() || it->second->state >= GS_REQ_DONE;
    };
    if(wait_ms < 0) done_cv_.wait(l, ended);
    else if(wait_ms > 0) done_cv_.wait_for(l, std::chrono::milliseconds(wait_ms), ended);
    auto it = reqs_.find(id);
    if(it == reqs_.end()) {
      err = "unknown request id";
      return GS_ERR_USAGE;
    }
    Request &r = *it->second;
    if(info) {
      info->state = r.state;
      info->status = r.status;
      info->patterns = r.patterns;
      const clk::time_point now = clk::now();
      info->queue_ms = r.state == GS_REQ_QUEUED ? ms_between(r.t_submit, now) : ms_between(r.t_submit, r.t_admit);
      info->latency_ms = r.state >= GS_REQ_DONE ? ms_between(r.t_submit, r.t_end) : 0.0;
      info->peak_bytes = r.peak_bytes;
    }
    if(r.state < GS_REQ_DONE) {
      err = "request still queued or running";
      return GS_ERR_TIMEOUT;
    }
    if(out) {
      *out = nullptr;
      if(r.state == GS_REQ_DONE && r.out) *out = r.out.release()->publish();
      reqs_.erase(it);
    }
    return GS_OK;
  }

  gs_status cancel(int64_t id, std::string &err)
  {
    std::lock_guard<std::mutex> g(m_);
    auto it = reqs_.find(id);
    if(it == reqs_.end()) {
      err = "unknown request id";
      return GS_ERR_USAGE;
    }
    if(it->second->state < GS_REQ_DONE) {
      it->second->cancel = true;
      cv_.notify_all();
    }
    return GS_OK;
  }

  void stats(gs_server_stats *s)
  {
    std::lock_guard<std::mutex> g(m_);
    std::memset(s, 0, sizeof(*s));
    s->submitted = submitted_;
    s->completed = completed_;
    s->cancelled = cancelled_;
    s->failed = failed_;
    s->queued = (int64_t)queue_.size();
    s->running = (int64_t)running_.size();
    s->max_running = max_running_;
    s->patterns = patterns_;
    std::vector<double> lat = latencies_;
    std::sort(lat.begin(), lat.end());
    auto rank = [&](double q) {
      // nearest rank: the smallest value with at least q of the samples at or below it
      size_t k = (size_t)std::ceil(q * (double)lat.size());
      if(k < 1) k = 1;
      return lat[std::min(lat.size(), k) - 1];
    };
    if(!lat.empty()) {
      s->p50_ms = rank(0.50);
      s->p99_ms = rank(0.99);
      double sum = 0;
      for(double v : lat) sum += v;
      s->mean_ms = sum / (double)lat.size();
    }
    s->wall_ms = ms_between(t_create_, clk::now());
    s->busy_ms = busy_ms_;
    s->budget_bytes = budget_;
    s->reserved_bytes = reserved_;
    s->pool_used_bytes = pool_used_;
    s->peak_pool_bytes = peak_pool_;
    s->waves = waves_;
    s->launches = launches_;
  }

private:
  gs_server_opts opt_;
  std::thread th_;
  std::mutex m_;
  std::condition_variable cv_, done_cv_;
  bool stop_ = false;
  std::vector<Database *> dbs_;
  std::unordered_map<int64_t, std::unique_ptr<Request>> reqs_;
  std::deque<int64_t> queue_;            // waiting for admission, arrival order
  std::vector<int64_t> running_;
  std::map<HistKey, int64_t> hist_;      // observed peak embedding-store bytes
  int64_t next_id_ = 1;
  int64_t submitted_ = 0, completed_ = 0, cancelled_ = 0, failed_ = 0, max_running_ = 0, patterns_ = 0;
  std::vector<double> latencies_;
  double busy_ms_ = 0;
  int64_t budget_ = 0, reserved_ = 0, pool_used_ = 0, peak_pool_ = 0, waves_ = 0, launches_ = 0;
  clk::time_point t_create_;
  // owned by the server thread
  std::unique_ptr<Scheduler> sched_;
  MineOptions wo_;
  std::unordered_map<int32_t, int64_t> job_req_;  // scheduler job -> request

  int64_t estimate(const Request &r) const
  {
    auto it = hist_.find(HistKey{ r.db_id, r.minsup, r.max_edges });
    if(it != hist_.end()) return it->second;
    return 20 * dbs_[r.db_id]->n_adj();
  }

  // under m_: end a request
  void end(Request &r, int32_t state, gs_status st, clk::time_point now)
  {
    r.state = state;
    r.status = st;
    r.t_end = now;
    if(state == GS_REQ_DONE) {
      completed_++;
      patterns_ += r.patterns;
      latencies_.push_back(ms_between(r.t_submit, r.t_end));
    } else if(state == GS_REQ_CANCELLED) {
      cancelled_++;
      r.out.reset();
    } else {
      failed_++;
      r.out.reset();
    }
  }

  void ensure_scheduler()
  {
    if(sched_) return;
    wo_ = MineOptions();
    if(opt_.wave_nodes > 0) wo_.wave_nodes = opt_.wave_nodes;
    if(opt_.threads > 0) wo_.threads = opt_.threads;
    wo_.extension = opt_.extension == GS_EXTENSION_LISTS ? 1 : opt_.extension == GS_EXTENSION_AUTO ? 2 : 0;
    sched_.reset(new Scheduler(wo_, opt_.pool_bytes));
    budget_ = opt_.budget_bytes;
    if(budget_ <= 0) {
      size_t freeb = 0, totalb = 0;
      if(cudaMemGetInfo(&freeb, &totalb) != cudaSuccess) {
        cudaGetLastError();
        freeb = 0;
      }
      budget_ = (int64_t)(freeb / 2);
    }
  }

  // the scheduler failed: every running request fails with the error
  void fail_running(gs_status st, const std::string &msg)
  {
    (void)msg;
    const clk::time_point now = clk::now();
    {
      std::lock_guard<std::mutex> g(m_);
      for(int64_t id : running_) {
        auto it = reqs_.find(id);
        if(it != reqs_.end()) end(*it->second, GS_REQ_FAILED, st, now);
      }
      running_.clear();
      reserved_ = 0;
    }
    job_req_.clear();
    try {
      if(sched_) sched_->reset();
    } catch(const Error &) {
      sched_.reset();
    }
    done_cv_.notify_all();
  }

  void loop()
  {
    while(true) {
      std::vector<std::pair<int64_t, MineJob>> admit;
      std::vector<int32_t> cancel_jobs;
      {
        std::unique_lock<std::mutex> l(m_);
        cv_.wait(l, [&] { return stop_ || !queue_.empty() || !running_.empty(); });
        if(stop_ && running_.empty()) {
          const clk::time_point now = clk::now();
          for(int64_t id : queue_) end(*reqs_[id], GS_REQ_CANCELLED, GS_ERR_CANCELLED, now);
          queue_.clear();
          done_cv_.notify_all();
          break;
        }
        const clk::time_point now = clk::now();
        // cancellations of queued requests end them now; running ones stop in the scheduler
        for(auto it = queue_.begin(); it != queue_.end();) {
          Request &r = *reqs_[*it];
          if(r.cancel) {
            end(r, GS_REQ_CANCELLED, GS_ERR_CANCELLED, now);
            it = queue_.erase(it);
          } else {
            ++it;
          }
        }
        for(int64_t id : running_) {
          Request &r = *reqs_[id];
          if(r.cancel && r.job >= 0) cancel_jobs.push_back(r.job);
        }
        // admission, arrival order: active slots and the embedding-store budget
        if(!stop_ && !queue_.empty() && !sched_) {
          // the scheduler (and the GPU context) is made on this thread at the first admission
          gs_status fail = GS_OK;
          try {
            ensure_scheduler();
          } catch(const Error &e) {
            fail = e.code;
          } catch(const std::exception &) {
            fail = GS_ERR_STATE;
          }
          if(fail != GS_OK) {
            sched_.reset();
            for(int64_t id : queue_) end(*reqs_[id], GS_REQ_FAILED, fail, now);
            queue_.clear();
            done_cv_.notify_all();
          }
        }
        while(!stop_ && !queue_.empty() && (int32_t)running_.size() < opt_.max_active) {
          Request &r = *reqs_[queue_.front()];
          const int64_t est = estimate(r);
          if(!running_.empty() && reserved_ + est > budget_) break;
          queue_.pop_front();
          r.state = GS_REQ_RUNNING;
          r.t_admit = now;
          r.estimate = est;
          reserved_ += est;
          r.out.reset(new PatternBuf());
          running_.push_back(r.id);
          max_running_ = std::max<int64_t>(max_running_, (int64_t)running_.size());
          MineJob j;
          j.db = dbs_[r.db_id];
          j.minsup = r.minsup;
          j.opt = wo_;
          j.opt.max_edges = r.max_edges;
          j.opt.label_style = opt_.label_style;
          j.emit = PatternBuf::emit;
          j.user = r.out.get();
          admit.emplace_back(r.id, j);
        }
        if(stop_)
          for(int64_t id : running_) {
            Request &r = *reqs_[id];
            if(r.job >= 0) cancel_jobs.push_back(r.job);
          }
      }
      if(!sched_) continue;
      const clk::time_point t0 = clk::now();
      try {
        for(int32_t jid : cancel_jobs) sched_->cancel(jid);
        for(auto &a : admit) {
          const int32_t jid = sched_->add(a.second);
          job_req_[jid] = a.first;
          std::lock_guard<std::mutex> g(m_);
          reqs_[a.first]->job = jid;
        }
        if(!sched_->idle()) sched_->step();
        retire();
      } catch(const Error &e) {
        fail_running(e.code, e.what());
      } catch(const std::exception &e) {
        fail_running(GS_ERR_STATE, e.what());
      }
      std::lock_guard<std::mutex> g(m_);
      busy_ms_ += ms_between(t0, clk::now());
    }
    sched_.reset();
  }

  // publishes the jobs the last step finished
  void retire()
  {
    std::vector<int32_t> done = sched_->take_done();
    if(done.empty()) {
      std::lock_guard<std::mutex> g(m_);
      pool_used_ = sched_->pool_used();
      return;
    }
    const clk::time_point now = clk::now();
    MineStats &st = sched_->stats();
    {
      std::lock_guard<std::mutex> g(m_);
      for(int32_t jid : done) {
        auto jr = job_req_.find(jid);
        if(jr == job_req_.end()) continue;
        JobInfo info;
        sched_->job_info(jid, info);
        sched_->forget(jid);
        auto it = reqs_.find(jr->second);
        job_req_.erase(jr);
        if(it == reqs_.end()) continue;
        Request &r = *it->second;
        running_.erase(std::find(running_.begin(), running_.end(), r.id));
        reserved_ -= r.estimate;
        r.patterns = info.patterns;
        r.peak_bytes = info.peak_bytes;
        if(info.cancelled) {
          end(r, GS_REQ_CANCELLED, GS_ERR_CANCELLED, now);
        } else {
          hist_[HistKey{ r.db_id, r.minsup, r.max_edges }] = std::max<int64_t>(info.peak_bytes, 1);
          end(r, GS_REQ_DONE, GS_OK, now);
        }
      }
      pool_used_ = sched_->pool_used();
      peak_pool_ = std::max<int64_t>(peak_pool_, pool_used_);
      waves_ = st.waves;
      launches_ = st.launches;
    }
    done_cv_.notify_all();
  }
};

}  // namespace gsgb

struct gs_server {
  std::unique_ptr<gsgb::Server> s;
};

extern "C" {

void gs_server_opts_default(gs_server_opts *o)
{
  if(!o) return;
  std::memset(o, 0, sizeof(*o));
  o->max_active = 64;
  o->label_style = GS_LABELS_FULL;
}

gs_status gs_server_create(const gs_server_opts *opts, gs_server **out)
{
  if(!out) {
    gsgb::capi_set_error("null output");
    return GS_ERR_USAGE;
  }
  gs_server_opts o;
  gs_server_opts_default(&o);
  if(opts) o = *opts;
  if(o.label_style != GS_LABELS_FULL && o.label_style != GS_LABELS_SEQ) {
    gsgb::capi_set_error("unknown label style");
    return GS_ERR_USAGE;
  }
  if(o.extension != GS_EXTENSION_RMPATH && o.extension != GS_EXTENSION_LISTS && o.extension != GS_EXTENSION_AUTO) {
    gsgb::capi_set_error("unknown extension strategy");
    return GS_ERR_USAGE;
  }
  gs_server *s = new gs_server();
  s->s.reset(new gsgb::Server(o));
  *out = s;
  return GS_OK;
}

gs_status gs_server_add_db(gs_server *srv, gs_db *db, int32_t *db_id)
{
  if(!srv || !db || !db_id) {
    gsgb::capi_set_error("null argument");
    return GS_ERR_USAGE;
  }
  *db_id = srv->s->add_db(&db->d);
  return GS_OK;
}

gs_status gs_server_submit(gs_server *srv, int32_t db_id, int32_t abs_minsup, int32_t max_edges,
                           int64_t *request_id)
{
  if(!srv || !request_id) {
    gsgb::capi_set_error("null argument");
    return GS_ERR_USAGE;
  }
  std::string err;
  gs_status st = srv->s->submit(db_id, abs_minsup, max_edges, request_id, err);
  if(st != GS_OK) gsgb::capi_set_error(err.c_str());
  return st;
}

gs_status gs_server_poll(gs_server *srv, int64_t request_id, int32_t wait_ms, gs_request_info *info,
                         gs_patterns **out)
{
  if(!srv) {
    gsgb::capi_set_error("null server");
    return GS_ERR_USAGE;
  }
  std::string err;
  gs_status st = srv->s->poll(request_id, wait_ms, info, out, err);
  if(st != GS_OK) gsgb::capi_set_error(err.c_str());
  return st;
}

gs_status gs_server_cancel(gs_server *srv, int64_t request_id)
{
  if(!srv) {
    gsgb::capi_set_error("null server");
    return GS_ERR_USAGE;
  }
  std::string err;
  gs_status st = srv->s->cancel(request_id, err);
  if(st != GS_OK) gsgb::capi_set_error(err.c_str());
  return st;
}

gs_status gs_server_get_stats(gs_server *srv, gs_server_stats *stats)
{
  if(!srv || !stats) {
    gsgb::capi_set_error("null argument");
    return GS_ERR_USAGE;
  }
  srv->s->stats(stats);
  return GS_OK;
}

void gs_server_destroy(gs_server *srv) { delete srv; }

}  // extern "C"
