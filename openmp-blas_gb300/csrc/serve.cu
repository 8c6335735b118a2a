// serve.cu - request loop with continuous batching (gbblas_server_*).
//
// Threads:
//   callers    gbblas_server_submit (any thread) appends to the pending FIFO;
//   scheduler  one native thread: admits pending requests in arrival order
//              while their working set fits the HBM budget and one of the
//              `streams` slots is free, coalesces the admitted ones into a
//              round - tensor-core GEMMs in one grouped launch per mode,
//              float GEMVs in one grouped launch, FP64 / FMA GEMMs and dots
//              as their own kernels - and enqueues the round on a free
//              stream followed by a host function;
//   CUDA       the host function runs when the round's work is done, stamps
//              its requests complete and hands the round back.
// Rounds on different streams overlap on the device; a request that arrives
// while others run joins the next round as soon as a slot and memory free up.
// Operands come from a CUDA memory pool owned by the server (kept resident).
#include <algorithm>
#include <cmath>
#include <atomic>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <thread>
#include <utility>
#include <vector>

#include "common.cuh"

namespace gbblas {

gbblas_status launch_gemv_group_rows_fixed(DeviceCtx* c, const gbblas_gemv_desc* d, int64_t count, cudaStream_t s,
                                           int R);

namespace {

using Clock = std::chrono::steady_clock;

struct Req {
  gbblas_request r{};
  int64_t bytes = 0;
  double est_us = 0.0;  // estimated GPU time
  bool heavy = false;
  int f64_digits = 0;         // double GEMM on tensor-core digits (0: the FP64 pipes)
  bool f64_guarded = false;   // ... in the guarded form
  Clock::time_point t_submit, t_round, t_enqueued, t_done;
  int round_size = 0;
  bool done = false;
  gbblas_status status = GBBLAS_STATUS_SUCCESS;
};

struct Round {
  void* srv = nullptr;  // the owning gbblas_server_s
  std::vector<Req*> reqs;
  int64_t bytes = 0;
  int stream_slot = 0;
  bool heavy = false;
  int max_ctas = 0;  // grid cap for the round's GEMMs (0 = whole GPU)
  int slices = 1;    // a heavy GEMM's launches over consecutive tile ranges
  gbblas_status status = GBBLAS_STATUS_SUCCESS;
};

int64_t round_up64(int64_t a, int64_t b) { return (a + b - 1) / b * b; }

// Tensor-core mode of an FP32 GEMM request that does not ask for the FMA
// path (AUTO: the FP32-accurate split-FP16 GEMM with its guard).
int server_mode(int32_t acc) {
  return acc == GBBLAS_ACCURACY_AUTO ? kTcModeF16Guard : tc_mode((gbblas_accuracy)acc);
}

// An AUTO float GEMM below 2^26 multiply-adds (about 400^3) runs as one FP32
// FMA kernel: the guarded split-FP16 chain is five launches (clears,
// exponents, pieces, GEMM, guard fix-up) whose fixed cost exceeds the whole
// FMA kernel at that size, and FMA arithmetic is FP32-accurate by
// definition.  The choice depends on the shape alone, so a request computes
// the same bits alone and in a mix.
constexpr double kServeAutoFmaMacs = 67108864.0;
bool server_auto_fma(const gbblas_request& r) {
  return r.op == GBBLAS_OP_MTM && r.dtype == GBBLAS_F32 && r.accuracy == GBBLAS_ACCURACY_AUTO &&
         (double)r.M * (double)r.N * (double)r.K < kServeAutoFmaMacs;
}

// Tensor-core digits of a double GEMM request (0: the FP64 pipes): FP64 means
// the pipes, FP64_DIGITS7 / 8 those digits, anything else (the float-only
// modes included) the library default - gbblas_dgemm's guarded 7-digit
// scheme where the shape suits.
int server_f64_digits(const gbblas_request& r, int sms, bool* guarded) {
  *guarded = false;
  if (r.op != GBBLAS_OP_MTM || r.dtype != GBBLAS_F64) return 0;
  if (const int d = dgemm_digits_count((gbblas_accuracy)r.accuracy)) return d;
  if (r.accuracy != GBBLAS_ACCURACY_FP64 && dgemm_auto_digits(r.M, r.N, r.K, sms)) {
    *guarded = true;
    return 7;
  }
  return 0;
}

// Device bytes a request holds while in flight: operands, result, and the
// operand arena (BF16 pieces or FP8 values and scales) of a tensor-core GEMM.
int64_t working_set(const gbblas_request& r, int f64_digits, bool f64_guarded) {
  const int64_t s = r.dtype == GBBLAS_F64 ? 8 : 4;
  switch (r.op) {
    case GBBLAS_OP_MTM: {
      int64_t b = (r.M * r.K + r.K * r.N + r.M * r.N) * s;
      if (r.dtype == GBBLAS_F32 && r.accuracy != GBBLAS_ACCURACY_FP32 && !server_auto_fma(r))
        b += (int64_t)tc_arena_bytes(server_mode(r.accuracy), r.M, r.N, r.K);
      if (f64_digits) b += (int64_t)dgemm_digits_scratch_bytes(f64_digits, f64_guarded, r.M, r.N, r.K);
      return b;
    }
    case GBBLAS_OP_MTV:
    case GBBLAS_OP_VTM:
      return (r.M * r.N + r.M + r.N) * s;
    default:
      return 2 * r.M * s + s;
  }
}

// Estimated GPU time (us) of a request from its flops / bytes and the rate of
// the path it takes on a GB300 (split-BF16 GEMM ~260 / ~430 TFLOP/s, split-FP16
// ~400, FP8 ~600, FP32 FMA ~55, FP64 pipes ~1.2 TFLOP/s, FP64 as tensor-core digits
// ~38 TFLOP/s after ~50 us of operand preparation and launches; streaming
// ~6 TB/s; FP64 GEMV ~1.1 TFLOP/s).
double estimate_us(const gbblas_request& r, int f64_digits) {
  const double launch = 5.0;
  switch (r.op) {
    case GBBLAS_OP_MTM: {
      const double fl = 2.0 * (double)r.M * (double)r.N * (double)r.K;
      double rate;  // flop per us
      if (f64_digits) return 50.0 + fl / 38e6;
      if (r.dtype == GBBLAS_F64)
        rate = 1.2e6;
      else if (r.accuracy == GBBLAS_ACCURACY_FP32)
        rate = 55e6;
      else if (server_auto_fma(r))
        rate = 20e6;  // the FMA kernel on shapes below 2^26 multiply-adds
      else if (r.accuracy == GBBLAS_ACCURACY_BF16X3)
        rate = 430e6;
      else if (r.accuracy == GBBLAS_ACCURACY_FP8)
        rate = 600e6;
      else if (r.accuracy == GBBLAS_ACCURACY_BF16X6)
        rate = 260e6;
      else  // split-FP16, AUTO's guarded split-FP16
        rate = 400e6;
      return launch + fl / rate;
    }
    case GBBLAS_OP_MTV:
    case GBBLAS_OP_VTM: {
      const double mn = (double)r.M * (double)r.N;
      return launch + (r.dtype == GBBLAS_F64 ? std::max(mn * 8 / 6e6, 2 * mn / 1.1e6) : mn * 4 / 6e6);
    }
    default:
      return launch + 2.0 * (double)r.M * (r.dtype == GBBLAS_F64 ? 8 : 4) / 6e6;
  }
}

}  // namespace
}  // namespace gbblas

using namespace gbblas;

struct gbblas_server_s {
  DeviceCtx* ctx = nullptr;
  int device = 0;
  gbblas_server_config cfg{};
  cudaMemPool_t pool = nullptr;
  cudaStream_t alloc_stream = nullptr;
  std::vector<cudaStream_t> streams;        // light rounds, high priority
  std::vector<bool> slot_busy;
  std::vector<cudaStream_t> heavy_streams;  // heavy requests, low priority
  std::vector<bool> heavy_busy;

  std::mutex mu;
  std::condition_variable cv;       // scheduler wake-ups
  std::condition_variable cv_done;  // waiters
  std::deque<Req*> pending;        // light requests, arrival order
  std::deque<Req*> heavy_pending;  // heavy requests, arrival order
  std::vector<std::unique_ptr<Req>> all;  // ticket -> request
  std::vector<Round*> finished;
  int inflight_rounds = 0;
  int inflight_heavy = 0;
  int64_t inflight_bytes = 0;
  bool budget_blocked = false;
  bool stop = false;
  std::thread scheduler;
  gbblas_server_stats stats{};
  int64_t round_reqs_total = 0;
  // host-side failure injection (gbblas_server_inject): events left to fail
  std::atomic<int> inject_alloc{0}, inject_launch{0};
};

namespace {

void CUDART_CB on_round_done(void* p) {
  Round* rd = static_cast<Round*>(p);
  const auto now = Clock::now();
  gbblas_server_s* s = static_cast<gbblas_server_s*>(rd->srv);
  {
    std::lock_guard<std::mutex> lk(s->mu);
    for (Req* q : rd->reqs) q->t_done = now;
    s->finished.push_back(rd);
  }
  s->cv.notify_one();
}

// Enqueue one round on `st` (scheduler thread, no lock held).
gbblas_status launch_round(gbblas_server_s* s, Round* rd, cudaStream_t st) {
  DeviceCtx* c = s->ctx;
  const int cap = rd->max_ctas;
  // tensor-core GEMMs of the round, one grouped launch per mode
  std::vector<std::pair<int, std::vector<gbblas_gemm_desc>>> groups;
  std::vector<gbblas_gemv_desc> gemv;
  gbblas_status first_err = GBBLAS_STATUS_SUCCESS;
  auto note = [&](gbblas_status e) {
    if (e != GBBLAS_STATUS_SUCCESS && first_err == GBBLAS_STATUS_SUCCESS) first_err = e;
  };
  for (Req* q : rd->reqs) {
    const gbblas_request& r = q->r;
    const bool row = r.layout == GBBLAS_LAST_ORDER;
    if (r.op == GBBLAS_OP_MTM) {
      const int64_t rsa = row ? r.K : 1, csa = row ? 1 : r.M, rsb = row ? r.N : 1, csb = row ? 1 : r.K,
                    rsc = row ? r.N : 1, csc = row ? 1 : r.M;
      if (q->f64_digits) {
        note(launch_dgemm_digits(c, q->f64_digits, q->f64_guarded, r.M, r.N, r.K,
                                 static_cast<const double*>(r.A), rsa, csa, static_cast<const double*>(r.B), rsb, csb,
                                 static_cast<double*>(r.C), rsc, csc, st, cap, rd->slices));
      } else if (r.dtype == GBBLAS_F64) {
        note(launch_gemm_fma<double>(c, r.M, r.N, r.K, static_cast<const double*>(r.A), rsa, csa,
                                     static_cast<const double*>(r.B), rsb, csb, static_cast<double*>(r.C), rsc,
                                     csc, st, cap));
      } else if (r.accuracy == GBBLAS_ACCURACY_FP32 || server_auto_fma(r)) {
        note(launch_gemm_fma<float>(c, r.M, r.N, r.K, static_cast<const float*>(r.A), rsa, csa,
                                    static_cast<const float*>(r.B), rsb, csb, static_cast<float*>(r.C), rsc, csc,
                                    st, cap));
      } else {
        gbblas_gemm_desc d{r.M, r.N, r.K, static_cast<const float*>(r.A), rsa, csa, static_cast<const float*>(r.B),
                           rsb, csb, static_cast<float*>(r.C), rsc, csc};
        const int mode = server_mode(r.accuracy);
        auto g = std::find_if(groups.begin(), groups.end(), [&](const auto& x) { return x.first == mode; });
        if (g == groups.end()) g = groups.insert(groups.end(), {mode, {}});
        g->second.push_back(d);
      }
    } else if (r.op == GBBLAS_OP_MTV || r.op == GBBLAS_OP_VTM) {
      const bool tr = r.op == GBBLAS_OP_VTM;
      // amt::mtv: column-major accumulates; amt::vtm: row-major accumulates
      const bool acc = tr ? row : !row;
      if (r.dtype == GBBLAS_F32) {
        gbblas_gemv_desc d{r.layout, tr ? 1 : 0, acc ? 1 : 0, 0, r.M, r.N, static_cast<const float*>(r.A),
                           static_cast<const float*>(r.B), static_cast<float*>(r.C)};
        gemv.push_back(d);
      } else {
        const int64_t out_len = tr ? r.N : r.M, red_len = tr ? r.M : r.N, lda = row ? r.N : r.M;
        const bool rows_contig = row != tr;
        const double* A = static_cast<const double*>(r.A);
        const double* x = static_cast<const double*>(r.B);
        double* y = static_cast<double*>(r.C);
        note(rows_contig ? launch_gemv_rows<double>(c, out_len, red_len, A, lda, x, y, acc, st)
                         : launch_gemv_cols<double>(c, out_len, red_len, A, lda, x, y, acc, st));
      }
    } else {
      if (r.dtype == GBBLAS_F64)
        note(launch_dot<double>(c, r.M, static_cast<const double*>(r.A), static_cast<const double*>(r.B),
                                static_cast<double*>(r.C), st));
      else
        note(launch_dot<float>(c, r.M, static_cast<const float*>(r.A), static_cast<const float*>(r.B),
                               static_cast<float*>(r.C), st));
    }
  }
  for (const auto& g : groups)
    note(launch_gemm_tc_group(c, g.first, g.second.data(), (int64_t)g.second.size(), st, cap, rd->slices));
  // fixed rows-per-item: no autotuning (timing) inside the serving loop
  if (!gemv.empty()) note(launch_gemv_group_rows_fixed(c, gemv.data(), (int64_t)gemv.size(), st, 4));
  rd->status = first_err;
  cudaError_t e = cudaLaunchHostFunc(st, on_round_done, rd);
  if (e != cudaSuccess) {
    set_error("server: cudaLaunchHostFunc failed: %s", cudaGetErrorString(e));
    return GBBLAS_STATUS_CUDA_ERROR;
  }
  return GBBLAS_STATUS_SUCCESS;
}

void scheduler_main(gbblas_server_s* s) {
  cudaSetDevice(s->device);
  std::unique_lock<std::mutex> lk(s->mu);
  auto light_ready = [&] {
    return !s->pending.empty() && s->inflight_rounds < (int)s->streams.size() && !s->budget_blocked;
  };
  auto heavy_ready = [&] {
    return !s->heavy_pending.empty() && s->inflight_heavy < (int)s->heavy_streams.size() && !s->budget_blocked;
  };
  for (;;) {
    s->cv.wait(lk, [&] {
      return !s->finished.empty() || light_ready() || heavy_ready() ||
             (s->stop && s->pending.empty() && s->heavy_pending.empty() && s->inflight_rounds == 0 &&
              s->inflight_heavy == 0);
    });
    // completions: release memory and slots, wake waiters
    if (!s->finished.empty()) {
      for (Round* rd : s->finished) {
        s->inflight_bytes -= rd->bytes;
        if (rd->heavy) {
          s->inflight_heavy--;
          s->heavy_busy[rd->stream_slot] = false;
        } else {
          s->inflight_rounds--;
          s->slot_busy[rd->stream_slot] = false;
        }
        for (Req* q : rd->reqs) {
          q->status = rd->status;
          q->done = true;
        }
        s->stats.completed += (int64_t)rd->reqs.size();
        delete rd;
      }
      s->finished.clear();
      s->budget_blocked = false;
      s->cv_done.notify_all();
    }
    if (s->stop && s->pending.empty() && s->heavy_pending.empty() && s->inflight_rounds == 0 &&
        s->inflight_heavy == 0)
      break;
    // Form rounds while slots are free.  Light rounds take requests in
    // arrival order up to max_group and up to heavy_us of estimated work;
    // a heavy request is a round by itself.
    bool progress = true;
    while (progress) {
      progress = false;
      for (int kind = 0; kind < 2; ++kind) {
        const bool heavy = kind == 1;
        std::deque<Req*>& q = heavy ? s->heavy_pending : s->pending;
        const int cap = heavy ? (int)s->heavy_streams.size() : (int)s->streams.size();
        int& inflight = heavy ? s->inflight_heavy : s->inflight_rounds;
        if (q.empty() || inflight >= cap || s->budget_blocked) continue;
        Round* rd = new Round();
        rd->srv = s;
        rd->heavy = heavy;
        double est = 0.0;
        while (!q.empty() && (int)rd->reqs.size() < (heavy ? 1 : s->cfg.max_group)) {
          Req* r = q.front();
          if (s->inflight_bytes + r->bytes > s->cfg.budget_bytes) break;  // wait for memory
          if (!rd->reqs.empty() && est + r->est_us > (double)s->cfg.heavy_us) break;
          q.pop_front();
          rd->reqs.push_back(r);
          rd->bytes += r->bytes;
          est += r->est_us;
          s->inflight_bytes += r->bytes;
        }
        if (rd->reqs.empty()) {
          delete rd;
          s->budget_blocked = true;
          continue;
        }
        std::vector<bool>& busy = heavy ? s->heavy_busy : s->slot_busy;
        int slot = 0;
        while (busy[slot]) ++slot;
        busy[slot] = true;
        rd->stream_slot = slot;
        inflight++;
        s->stats.rounds++;
        s->round_reqs_total += (int64_t)rd->reqs.size();
        if (s->inflight_bytes > s->stats.peak_inflight_bytes) s->stats.peak_inflight_bytes = s->inflight_bytes;
        // A heavy round's CTAs run for milliseconds and are not preempted by
        // higher-priority streams, and light requests that arrive after it
        // started would find every SM taken: a heavy round's grid is capped
        // at three quarters of the SMs, so light rounds always keep a quarter
        // of the GPU.  (Capping only while light work was already queued let
        // later arrivals wait behind whole heavy kernels: p99 2.3x the lone
        // p99 at 1 k req/s against 1.1x with the permanent cap.)
        if (heavy) {
          // A heavy tensor-core or digit GEMM runs on the whole GPU as slices
          // of about slice_us each: between slices the block scheduler serves
          // the high-priority light streams first.  Other heavy requests keep
          // the SM cap.
          Req* h = rd->reqs[0];
          const bool sliceable = h->r.op == GBBLAS_OP_MTM &&
                                 (h->f64_digits || (h->r.dtype == GBBLAS_F32 && h->r.accuracy != GBBLAS_ACCURACY_FP32));
          if (sliceable && s->cfg.slice_us > 0)
            rd->slices = (int)std::max(1.0, std::ceil(h->est_us / (double)s->cfg.slice_us));
          else
            rd->max_ctas = std::max(1, s->ctx->num_sms * s->cfg.heavy_sm_percent / 100);
        }
        cudaStream_t st = heavy ? s->heavy_streams[slot] : s->streams[slot];
        const auto t_round = Clock::now();
        for (Req* r : rd->reqs) {
          r->t_round = t_round;
          r->round_size = (int)rd->reqs.size();
        }
        lk.unlock();
        gbblas_status e;
        if (s->inject_launch.load() > 0 && s->inject_launch.fetch_sub(1) > 0) {
          set_error("server: injected launch failure");
          e = GBBLAS_STATUS_CUDA_ERROR;
        } else {
          e = launch_round(s, rd, st);
        }
        const auto t_enq = Clock::now();
        lk.lock();
        for (Req* r : rd->reqs) r->t_enqueued = t_enq;
        if (e != GBBLAS_STATUS_SUCCESS) {  // the host function never runs: finish here
          rd->status = e;
          for (Req* r : rd->reqs) {
            r->t_done = t_enq;
            r->round_size = 0;  // it never ran
          }
          s->finished.push_back(rd);
        }
        progress = true;
      }
    }
  }
}

}  // namespace

extern "C" {

gbblas_status gbblas_server_create(const gbblas_server_config* cfg, gbblas_server* out) {
  if (!out) {
    set_error("gbblas_server_create: null output");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  DeviceCtx* c;
  GB_TRY(get_ctx(&c));
  auto s = std::make_unique<gbblas_server_s>();
  s->ctx = c;
  s->device = c->device;
  // Defaults from the serving sweep at 10-40 k req/s on GB300 (60/30/10
  // mtm/mtv/dot): 16 light streams with 300 us of estimated work per light
  // round kept p99 within 1.24-1.31x of the lone p99 at 20 k req/s, against
  // 2.0-2.4x with 4 streams and 1000 us.
  s->cfg.streams = 16;
  s->cfg.max_group = 256;
  s->cfg.budget_bytes = int64_t(64) << 30;
  s->cfg.scratch_bytes = int64_t(1) << 30;
  s->cfg.heavy_streams = 2;
  s->cfg.heavy_us = 300;
  s->cfg.heavy_sm_percent = 75;
  s->cfg.slice_us = 200;
  if (cfg) {
    if (cfg->slice_us != 0) s->cfg.slice_us = cfg->slice_us;
    if (cfg->heavy_streams > 0) s->cfg.heavy_streams = cfg->heavy_streams;
    if (cfg->heavy_sm_percent > 0) s->cfg.heavy_sm_percent = std::min(cfg->heavy_sm_percent, 100);
    if (cfg->heavy_us > 0) s->cfg.heavy_us = cfg->heavy_us;
    if (cfg->streams > 0) s->cfg.streams = cfg->streams;
    if (cfg->max_group > 0) s->cfg.max_group = cfg->max_group;
    if (cfg->budget_bytes > 0) s->cfg.budget_bytes = cfg->budget_bytes;
    if (cfg->scratch_bytes > 0) s->cfg.scratch_bytes = cfg->scratch_bytes;
  }
  cudaMemPoolProps props{};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = c->device;
  GB_CUDA_TRY(cudaMemPoolCreate(&s->pool, &props));
  uint64_t keep = UINT64_MAX;  // never trim: operands stay resident
  GB_CUDA_TRY(cudaMemPoolSetAttribute(s->pool, cudaMemPoolAttrReleaseThreshold, &keep));
  GB_CUDA_TRY(cudaStreamCreateWithFlags(&s->alloc_stream, cudaStreamNonBlocking));
  tc_prepare(c);
  int prio_low = 0, prio_high = 0;  // numerically: low priority >= high priority
  GB_CUDA_TRY(cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high));
  for (int i = 0; i < s->cfg.streams + s->cfg.heavy_streams; ++i) {
    const bool heavy = i >= s->cfg.streams;
    cudaStream_t st;
    GB_CUDA_TRY(cudaStreamCreateWithPriority(&st, cudaStreamNonBlocking, heavy ? prio_low : prio_high));
    (heavy ? s->heavy_streams : s->streams).push_back(st);
    (heavy ? s->heavy_busy : s->slot_busy).push_back(false);
    void* scr = nullptr;
    GB_TRY(get_scratch(c, st, (size_t)s->cfg.scratch_bytes, &scr));
  }
  for (cudaStream_t st : s->streams) GB_CUDA_TRY(cudaStreamSynchronize(st));
  for (cudaStream_t st : s->heavy_streams) GB_CUDA_TRY(cudaStreamSynchronize(st));
  s->scheduler = std::thread(scheduler_main, s.get());
  *out = s.release();
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_server_alloc(gbblas_server s, int64_t bytes, void** ptr) {
  if (!s || !ptr || bytes < 0) {
    set_error("gbblas_server_alloc: bad arguments");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  if (s->inject_alloc.load() > 0 && s->inject_alloc.fetch_sub(1) > 0) {
    set_error("gbblas_server_alloc of %lld bytes failed: injected failure", (long long)bytes);
    return GBBLAS_STATUS_ALLOC_FAILED;
  }
  cudaError_t e = cudaMallocFromPoolAsync(ptr, (size_t)(bytes ? bytes : 1), s->pool, s->alloc_stream);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s->alloc_stream);
  if (e != cudaSuccess) {
    set_error("gbblas_server_alloc of %lld bytes failed: %s", (long long)bytes, cudaGetErrorString(e));
    return GBBLAS_STATUS_ALLOC_FAILED;
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_server_free(gbblas_server s, void* ptr) {
  if (!s) {
    set_error("gbblas_server_free: null server");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  if (!ptr) return GBBLAS_STATUS_SUCCESS;
  GB_CUDA_TRY(cudaFreeAsync(ptr, s->alloc_stream));
  GB_CUDA_TRY(cudaStreamSynchronize(s->alloc_stream));
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_server_submit(gbblas_server s, const gbblas_request* r, uint64_t* ticket) {
  if (!s || !r || !ticket) {
    set_error("gbblas_server_submit: bad arguments");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  if (r->op < GBBLAS_OP_MTM || r->op > GBBLAS_OP_DOT || (r->dtype != GBBLAS_F32 && r->dtype != GBBLAS_F64) ||
      (r->layout != GBBLAS_FIRST_ORDER && r->layout != GBBLAS_LAST_ORDER) || r->accuracy < 0 ||
      (r->dtype == GBBLAS_F64 ? r->accuracy > 7 : (r->accuracy > 4 && r->accuracy != GBBLAS_ACCURACY_FP16X3))) {
    set_error("gbblas_server_submit: bad op, dtype, layout or accuracy");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  if (r->M < 0 || r->N < 0 || r->K < 0 || !r->A || !r->B || !r->C) {
    set_error("gbblas_server_submit: negative size or null operand");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  auto q = std::make_unique<Req>();
  q->r = *r;
  q->f64_digits = server_f64_digits(*r, s->ctx->num_sms, &q->f64_guarded);
  q->bytes = working_set(*r, q->f64_digits, q->f64_guarded);
  q->est_us = estimate_us(*r, q->f64_digits);
  q->heavy = q->est_us > (double)s->cfg.heavy_us;
  if (q->bytes > s->cfg.budget_bytes) {
    set_error("gbblas_server_submit: request needs %lld bytes, the budget is %lld", (long long)q->bytes,
              (long long)s->cfg.budget_bytes);
    std::lock_guard<std::mutex> lk(s->mu);
    s->stats.rejected++;
    return GBBLAS_STATUS_ALLOC_FAILED;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    q->t_submit = Clock::now();
    *ticket = (uint64_t)s->all.size();
    (q->heavy ? s->heavy_pending : s->pending).push_back(q.get());
    s->all.push_back(std::move(q));
    s->stats.submitted++;
  }
  s->cv.notify_one();
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_server_wait(gbblas_server s, uint64_t ticket, double* latency_s) {
  if (!s) {
    set_error("gbblas_server_wait: null server");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  std::unique_lock<std::mutex> lk(s->mu);
  if (ticket >= s->all.size()) {
    set_error("gbblas_server_wait: unknown ticket");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  Req* q = s->all[ticket].get();
  s->cv_done.wait(lk, [&] { return q->done; });
  if (latency_s) latency_s[0] = std::chrono::duration<double>(q->t_done - q->t_submit).count();
  if (q->status != GBBLAS_STATUS_SUCCESS)
    set_error("gbblas_server: request %llu %s", (unsigned long long)ticket,
              q->status == GBBLAS_STATUS_CANCELLED ? "was cancelled" : "failed");
  return q->status;
}

gbblas_status gbblas_server_run_trace(gbblas_server s, const gbblas_request* reqs, const double* arrival_s, int64_t n,
                                      double* latency_s) {
  if (!s || n < 0 || (n > 0 && (!reqs || !arrival_s))) {
    set_error("gbblas_server_run_trace: bad arguments");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  std::vector<uint64_t> tickets((size_t)n);
  std::vector<gbblas_status> sub((size_t)n, GBBLAS_STATUS_SUCCESS);
  const auto t0 = Clock::now();
  std::thread submitter([&] {
    cudaSetDevice(s->device);
    for (int64_t i = 0; i < n; ++i) {
      const auto target = t0 + std::chrono::duration_cast<Clock::duration>(std::chrono::duration<double>(arrival_s[i]));
      if (Clock::now() + std::chrono::microseconds(200) < target)
        std::this_thread::sleep_until(target - std::chrono::microseconds(100));
      while (Clock::now() < target) {
      }
      sub[(size_t)i] = gbblas_server_submit(s, &reqs[i], &tickets[(size_t)i]);
    }
  });
  submitter.join();
  gbblas_status st = GBBLAS_STATUS_SUCCESS;
  for (int64_t i = 0; i < n; ++i) {
    double lat = -1.0;
    gbblas_status e = sub[(size_t)i];
    if (e == GBBLAS_STATUS_SUCCESS) e = gbblas_server_wait(s, tickets[(size_t)i], &lat);
    if (latency_s) latency_s[i] = e == GBBLAS_STATUS_SUCCESS ? lat : -1.0;
    if (e != GBBLAS_STATUS_SUCCESS && st == GBBLAS_STATUS_SUCCESS) st = e;
  }
  return st;
}

gbblas_status gbblas_server_get_stats(gbblas_server s, gbblas_server_stats* out) {
  if (!s || !out) {
    set_error("gbblas_server_get_stats: bad arguments");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  *out = s->stats;
  out->mean_round_size = s->stats.rounds ? (double)s->round_reqs_total / (double)s->stats.rounds : 0.0;
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_server_request_times(gbblas_server s, uint64_t ticket, double* times) {
  if (!s || !times) {
    set_error("gbblas_server_request_times: bad arguments");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  std::lock_guard<std::mutex> lk(s->mu);
  if (ticket >= s->all.size()) {
    set_error("gbblas_server_request_times: unknown ticket");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  const Req* q = s->all[ticket].get();
  if (!q->done) {
    set_error("gbblas_server_request_times: request %llu has not finished", (unsigned long long)ticket);
    return GBBLAS_STATUS_NOT_SUPPORTED;
  }
  auto sec = [](Clock::time_point a, Clock::time_point b) { return std::chrono::duration<double>(b - a).count(); };
  if (q->round_size == 0) {
    times[0] = times[1] = times[2] = times[3] = 0.0;
  } else {
    times[0] = sec(q->t_submit, q->t_round);
    times[1] = sec(q->t_round, q->t_enqueued);
    // the completion stamp can precede the enqueue stamp by the few
    // microseconds between the round's last launch and the scheduler's clock
    times[2] = std::max(0.0, sec(q->t_enqueued, q->t_done));
    times[3] = (double)q->round_size;
  }
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_server_cancel(gbblas_server s, uint64_t ticket) {
  if (!s) {
    set_error("gbblas_server_cancel: null server");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  {
    std::lock_guard<std::mutex> lk(s->mu);
    if (ticket >= s->all.size()) {
      set_error("gbblas_server_cancel: unknown ticket");
      return GBBLAS_STATUS_INVALID_VALUE;
    }
    Req* q = s->all[ticket].get();
    std::deque<Req*>& dq = q->heavy ? s->heavy_pending : s->pending;
    auto it = std::find(dq.begin(), dq.end(), q);
    if (it == dq.end()) {
      set_error("gbblas_server_cancel: request %llu already %s", (unsigned long long)ticket,
                q->done ? "finished" : "running");
      return GBBLAS_STATUS_NOT_SUPPORTED;
    }
    dq.erase(it);
    q->status = GBBLAS_STATUS_CANCELLED;
    q->t_done = Clock::now();
    q->done = true;
    // a queue head that waited for memory may have been this one
    s->budget_blocked = false;
  }
  s->cv_done.notify_all();
  s->cv.notify_one();
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_server_inject(gbblas_server s, int32_t kind, int32_t count) {
  if (!s || count < 0 || (kind != GBBLAS_INJECT_ALLOC && kind != GBBLAS_INJECT_LAUNCH)) {
    set_error("gbblas_server_inject: bad arguments");
    return GBBLAS_STATUS_INVALID_VALUE;
  }
  (kind == GBBLAS_INJECT_ALLOC ? s->inject_alloc : s->inject_launch).store(count);
  return GBBLAS_STATUS_SUCCESS;
}

gbblas_status gbblas_server_destroy(gbblas_server s) {
  if (!s) return GBBLAS_STATUS_SUCCESS;
  {
    std::lock_guard<std::mutex> lk(s->mu);
    s->stop = true;
  }
  s->cv.notify_all();
  if (s->scheduler.joinable()) s->scheduler.join();
  std::vector<cudaStream_t> all_streams = s->streams;
  all_streams.insert(all_streams.end(), s->heavy_streams.begin(), s->heavy_streams.end());
  for (cudaStream_t st : all_streams) {
    cudaStreamSynchronize(st);
    release_scratch(s->ctx, st);
    cudaStreamSynchronize(st);
    cudaStreamDestroy(st);
  }
  if (s->alloc_stream) {
    cudaStreamSynchronize(s->alloc_stream);
    cudaStreamDestroy(s->alloc_stream);
  }
  if (s->pool) cudaMemPoolDestroy(s->pool);
  delete s;
  return GBBLAS_STATUS_SUCCESS;
}

}  // extern "C"
