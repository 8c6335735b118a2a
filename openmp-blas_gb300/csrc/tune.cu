// tune.cu - the autotuner.
//
// The reference picks its blocking once per process from the CPU's cache
// geometry and a hard-coded FMA latency table (include/mtm.hpp:19-81,
// include/cpuinfo.hpp:167-223, include/cache_manager.hpp:107-150).  On the
// GPU the choices are kernel variants, and they are picked by measurement:
// the first time a (device, operation, shape bucket, dtype, accuracy) key is
// seen, every candidate is timed with CUDA events on scratch outputs and the
// fastest is remembered - in memory, and in a JSON file so later processes
// start tuned.
//
//   GBBLAS_AUTOTUNE=0      use the built-in defaults, time nothing
//   GBBLAS_TUNE_CACHE=path cache file (default $XDG_CACHE_HOME/gbblas/tune.json
//                          or ~/.cache/gbblas/tune.json); unwritable = memory only
//
// Tuned choices:
//   gemv_group_rows  rows per warp item of the grouped row-streaming GEMV
//                    (1, 2, 4, 8), bucketed by median log2 rows / cols;
//   gemm_auto        for GBBLAS_ACCURACY_AUTO, FP32 FMA kernel or the guarded
//                    FP16 split (three products) - both FP32-accurate -
//                    bucketed by log2 M, N, K;
//   gemm_tc          per tensor-core mode and log2 M, N, K bucket: split-K
//                    parts (1, 2, 4, 8, 16; offered when K >= 4 max(M, N) and
//                    the output tiles fill at most half the SMs) and the CTA
//                    form (single CTAs or CTA pairs, split-BF16 only);
//                    GBBLAS_TC_SPLITK=n forces n parts;
//   gemm_fma_tile    FP32 FMA kernel and CTA tile per bucket: 64 x 64 or
//                    128 x 128 register-staged, the TMA-fed 128 x 128, or
//                    that in stream-K form where whole tiles fill the SMs badly;
//                    GBBLAS_FMA_TILE=0 / 1 / 2 / 3 forces one.
// Nothing is timed while the caller's stream is being captured into a graph
// (the defaults apply); single-call paths consult the tuner, grouped,
// batched and served launches use the defaults.
#include <sys/stat.h>

#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <map>
#include <regex>
#include <sstream>
#include <string>
#include <vector>

#include "common.cuh"

namespace gbblas {

gbblas_status time_gemv_group_variant(DeviceCtx* c, const gbblas_gemv_desc* d, int64_t count, int R, float* ms);

namespace {

class Tuner {
 public:
  static Tuner& get() {
    static Tuner t;
    return t;
  }

  bool enabled() const { return enabled_; }

  // Cached choice for `key`, or -1.
  int lookup(const std::string& key) {
    std::lock_guard<std::mutex> lk(mu_);
    load_locked();
    auto it = cache_.find(key);
    return it == cache_.end() ? -1 : it->second;
  }

  void store(const std::string& key, int value) {
    std::lock_guard<std::mutex> lk(mu_);
    load_locked();
    cache_[key] = value;
    save_locked();
  }

 private:
  Tuner() {
    const char* e = std::getenv("GBBLAS_AUTOTUNE");
    enabled_ = !(e && std::string(e) == "0");
    if (const char* p = std::getenv("GBBLAS_TUNE_CACHE")) {
      path_ = p;
    } else if (const char* x = std::getenv("XDG_CACHE_HOME")) {
      path_ = std::string(x) + "/gbblas/tune.json";
    } else if (const char* h = std::getenv("HOME")) {
      path_ = std::string(h) + "/.cache/gbblas/tune.json";
    }
  }

  void load_locked() {
    if (loaded_) return;
    loaded_ = true;
    if (path_.empty()) return;
    std::ifstream f(path_);
    if (!f) return;
    std::stringstream ss;
    ss << f.rdbuf();
    const std::string text = ss.str();
    static const std::regex kv("\"([^\"]+)\"\\s*:\\s*(-?[0-9]+)");
    for (auto it = std::sregex_iterator(text.begin(), text.end(), kv); it != std::sregex_iterator(); ++it) {
      const std::string key = (*it)[1];
      if (key == "version") continue;
      cache_[key] = std::atoi((*it)[2].str().c_str());
    }
  }

  void save_locked() {
    if (path_.empty()) return;
    const auto slash = path_.find_last_of('/');
    if (slash != std::string::npos) {
      std::string dir = path_.substr(0, slash);
      for (size_t i = 1; i <= dir.size(); ++i)
        if (i == dir.size() || dir[i] == '/') ::mkdir(dir.substr(0, i).c_str(), 0755);
    }
    const std::string tmp = path_ + ".tmp";
    std::ofstream f(tmp);
    if (!f) return;
    f << "{\n  \"version\": 1";
    for (const auto& kv : cache_) f << ",\n  \"" << kv.first << "\": " << kv.second;
    f << "\n}\n";
    f.close();
    std::rename(tmp.c_str(), path_.c_str());
  }

  std::mutex mu_;
  std::map<std::string, int> cache_;
  bool loaded_ = false;
  bool enabled_ = true;
  std::string path_;
};

std::string device_tag(DeviceCtx* c) {
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, c->device) != cudaSuccess) return "unknown";
  std::string name = p.name;
  std::replace(name.begin(), name.end(), ' ', '_');
  return name + "_sm" + std::to_string(c->num_sms);
}

int log2_bucket(int64_t v) { return v <= 1 ? 0 : (int)std::lround(std::log2((double)v)); }

bool capturing(cudaStream_t s) {
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &st) != cudaSuccess) {
    cudaGetLastError();
    return true;  // unknown: do not time
  }
  return st != cudaStreamCaptureStatusNone;
}

// Scratch FP32 operands (zeros) for timing one GEMM shape on the tuner's own
// stream; each candidate runs once to warm up, then 3 times between events.
class GemmBench {
 public:
  GemmBench(DeviceCtx* c, int64_t m, int64_t n, int64_t k) : c_(c), m_(m), n_(n), k_(k) {
    if (cudaStreamCreateWithFlags(&s_, cudaStreamNonBlocking) != cudaSuccess) return;
    const size_t bytes = sizeof(float) * (size_t)(m * k + k * n + m * n);
    if (cudaMallocAsync(&mem_, bytes, s_) != cudaSuccess) {
      mem_ = nullptr;
      return;
    }
    cudaMemsetAsync(mem_, 0, bytes, s_);
    cudaEventCreate(&e0_);
    cudaEventCreate(&e1_);
  }
  ~GemmBench() {
    if (mem_) cudaFreeAsync(mem_, s_);
    if (s_) {
      cudaStreamSynchronize(s_);
      release_scratch(c_, s_);
      cudaStreamDestroy(s_);
    }
    if (e0_) cudaEventDestroy(e0_);
    if (e1_) cudaEventDestroy(e1_);
  }
  bool ok() const { return mem_ != nullptr; }
  gbblas_gemm_desc desc() const {
    float* A = static_cast<float*>(mem_);
    float* B = A + m_ * k_;
    float* C = B + k_ * n_;
    return gbblas_gemm_desc{m_, n_, k_, A, k_, 1, B, n_, 1, C, n_, 1};
  }
  cudaStream_t stream() const { return s_; }
  // ms per call of run(stream), or a huge value if it failed
  template <typename F>
  float time(F&& run) {
    if (run(s_) != GBBLAS_STATUS_SUCCESS) return 1e30f;
    cudaEventRecord(e0_, s_);
    for (int i = 0; i < 3; ++i)
      if (run(s_) != GBBLAS_STATUS_SUCCESS) return 1e30f;
    cudaEventRecord(e1_, s_);
    if (cudaEventSynchronize(e1_) != cudaSuccess) return 1e30f;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0_, e1_);
    return ms;
  }

 private:
  DeviceCtx* c_;
  int64_t m_, n_, k_;
  cudaStream_t s_ = nullptr;
  void* mem_ = nullptr;
  cudaEvent_t e0_ = nullptr, e1_ = nullptr;
};

// Representative shape of a log2 bucket: 2^b per dimension, M and N at most
// 8192, K at most 2^16, and the operands at most 2^28 elements.
void bucket_shape(int bm, int bn, int bk, int64_t& m, int64_t& n, int64_t& k) {
  m = std::min<int64_t>(int64_t(1) << bm, 8192);
  n = std::min<int64_t>(int64_t(1) << bn, 8192);
  k = std::min<int64_t>(int64_t(1) << bk, 65536);
  while ((m + n) * k > (int64_t(1) << 28) && k > 64) k >>= 1;
}

}  // namespace

int tuned_gemv_group_rows(DeviceCtx* c, const gbblas_gemv_desc* d, int64_t count) {
  constexpr int kDefault = 4;
  Tuner& t = Tuner::get();
  std::vector<int64_t> rows, cols;
  for (int64_t i = 0; i < count; ++i) {
    const bool tr = d[i].transpose != 0;
    const bool rows_contig = (d[i].layout == GBBLAS_LAST_ORDER) != tr;
    if (!rows_contig || d[i].M <= 0 || d[i].N <= 0) continue;
    rows.push_back(tr ? d[i].N : d[i].M);
    cols.push_back(tr ? d[i].M : d[i].N);
  }
  if (rows.empty()) return kDefault;
  std::nth_element(rows.begin(), rows.begin() + rows.size() / 2, rows.end());
  std::nth_element(cols.begin(), cols.begin() + cols.size() / 2, cols.end());
  const std::string key = "gemv_group_rows|" + device_tag(c) + "|r" + std::to_string(log2_bucket(rows[rows.size() / 2])) +
                          "|c" + std::to_string(log2_bucket(cols[cols.size() / 2])) + "|n" +
                          std::to_string(log2_bucket((int64_t)rows.size())) + "|f32";
  int v = t.lookup(key);
  if (v > 0) return v;
  if (!t.enabled()) return kDefault;
  int best = kDefault;
  float best_ms = 1e30f;
  for (int R : {1, 2, 4, 8}) {
    float ms = 0.f;
    if (time_gemv_group_variant(c, d, count, R, &ms) != GBBLAS_STATUS_SUCCESS) return kDefault;
    if (ms < best_ms) {
      best_ms = ms;
      best = R;
    }
  }
  t.store(key, best);
  return best;
}

// 1 = split-BF16 (six products), 0 = FP32 FMA, for an AUTO-accuracy GEMM of
// this shape.  Without tuning: the tensor cores once the work fills them.
int tuned_gemm_auto(DeviceCtx* c, int64_t M, int64_t N, int64_t K) {
  if (const char* e = std::getenv("GBBLAS_GEMM_AUTO"); e && (e[0] == '0' || e[0] == '1')) return e[0] - '0';
  const int fallback = (M >= 256 && N >= 256 && K >= 256 && (double)M * N * K >= 1.0e9) ? 1 : 0;
  Tuner& t = Tuner::get();
  const int bm = log2_bucket(M), bn = log2_bucket(N), bk = log2_bucket(K);
  const std::string key = "gemm_auto_f16g|" + device_tag(c) + "|m" + std::to_string(bm) + "|n" + std::to_string(bn) +
                          "|k" + std::to_string(bk) + "|f32";
  int v = t.lookup(key);
  if (v >= 0) return v;
  if (!t.enabled()) return fallback;
  // representative shape of the bucket, capped so tuning stays cheap
  const int64_t m = std::min<int64_t>(int64_t(1) << bm, 8192), n = std::min<int64_t>(int64_t(1) << bn, 8192),
                k = std::min<int64_t>(int64_t(1) << bk, 8192);
  cudaStream_t s;
  if (cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking) != cudaSuccess) return fallback;
  void* mem = nullptr;
  const size_t bytes = sizeof(float) * (size_t)(m * k + k * n + m * n);
  if (cudaMallocAsync(&mem, bytes, s) != cudaSuccess) {
    cudaStreamDestroy(s);
    return fallback;
  }
  cudaMemsetAsync(mem, 0, bytes, s);
  float* A = static_cast<float*>(mem);
  float* B = A + m * k;
  float* C = B + k * n;
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  float best_ms[2] = {1e30f, 1e30f};
  for (int choice = 0; choice < 2; ++choice) {
    auto run = [&]() {
      return choice == 1 ? launch_gemm_tc(c, kTcModeF16Guard, m, n, k, A, k, 1, B, n, 1, C, n, 1, s)
                         : launch_gemm_fma<float>(c, m, n, k, A, k, 1, B, n, 1, C, n, 1, s);
    };
    if (run() != GBBLAS_STATUS_SUCCESS) continue;  // warm-up
    cudaEventRecord(e0, s);
    bool ok = true;
    for (int i = 0; i < 3 && ok; ++i) ok = run() == GBBLAS_STATUS_SUCCESS;
    cudaEventRecord(e1, s);
    if (!ok || cudaEventSynchronize(e1) != cudaSuccess) continue;
    float ms = 0.f;
    cudaEventElapsedTime(&ms, e0, e1);
    best_ms[choice] = ms;
  }
  cudaFreeAsync(mem, s);
  cudaStreamSynchronize(s);
  release_scratch(c, s);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaStreamDestroy(s);
  if (best_ms[0] >= 1e30f && best_ms[1] >= 1e30f) return fallback;
  const int best = best_ms[1] < best_ms[0] ? 1 : 0;
  t.store(key, best);
  return best;
}

// Split-K parts worth trying for an M x N x K tensor-core GEMM: K at least
// four times the larger output side, output tiles filling at most half the
// SMs, every part at least 8 K stages, parts x tiles at most twice the SMs.
static std::vector<int> split_candidates(DeviceCtx* c, int mode, int64_t M, int64_t N, int64_t K) {
  std::vector<int> out;
  const int64_t tiles = ((M + 127) / 128) * ((N + 127) / 128);
  const int64_t stages = (K + tc_stage_k(mode) - 1) / tc_stage_k(mode);
  if (K < 4 * std::max(M, N) || 2 * tiles > c->num_sms) return out;
  for (int s : {2, 4, 8, 16})
    if (stages >= 8 * s && tiles * s <= 2 * (int64_t)c->num_sms) out.push_back(s);
  return out;
}

TcLaunchOpts tuned_tc_opts(DeviceCtx* c, int mode, int64_t M, int64_t N, int64_t K, cudaStream_t stream) {
  TcLaunchOpts def;
  if (const char* e = std::getenv("GBBLAS_TC_SPLITK"); e && std::atoi(e) > 0) {
    def.split = std::atoi(e);
    return def;
  }
  const std::vector<int> splits = split_candidates(c, mode, M, N, K);
  // GBBLAS_TC_PAIR, when set, fixes the CTA form; otherwise the tuner picks it
  // (pairs only where padding M to 256 rows adds at most 10 % of the work)
  const char* pe = std::getenv("GBBLAS_TC_PAIR");
  const bool pair_env = pe && pe[0];
  const int single = pair_env ? -1 : 0;
  const bool pairs = !pair_env && mode != tc_mode(GBBLAS_ACCURACY_FP8) && mode != tc_mode(GBBLAS_ACCURACY_FP16X3) &&
                     M >= 256 &&
                     (double)((M + 255) / 256 * 256) <= 1.1 * (double)((M + 127) / 128 * 128);
  // without measurements: the largest listed split (the tiles alone leave
  // most SMs idle) and the GBBLAS_TC_PAIR setting
  TcLaunchOpts fallback = def;
  if (!splits.empty()) fallback.split = splits.back();
  if (splits.empty() && !pairs) return def;
  Tuner& t = Tuner::get();
  const int bm = log2_bucket(M), bn = log2_bucket(N), bk = log2_bucket(K);
  const std::string key = "gemm_tc|" + device_tag(c) + "|mode" + std::to_string(mode) + "|m" + std::to_string(bm) +
                          "|n" + std::to_string(bn) + "|k" + std::to_string(bk);
  const int v = t.lookup(key);
  if (v >= 0) return TcLaunchOpts{std::max(1, v / 4), pair_env ? -1 : v % 4 - 1};
  if (!t.enabled() || capturing(stream)) return fallback;
  int64_t m, n, k;
  bucket_shape(bm, bn, bk, m, n, k);
  std::vector<TcLaunchOpts> cands{TcLaunchOpts{1, single}};
  for (int s : split_candidates(c, mode, m, n, k)) cands.push_back(TcLaunchOpts{s, single});
  if (pairs && m >= 256) cands.push_back(TcLaunchOpts{1, 1});
  if (cands.size() == 1) return fallback;
  GemmBench b(c, m, n, k);
  if (!b.ok()) return fallback;
  const gbblas_gemm_desc d = b.desc();
  TcLaunchOpts best = fallback;
  float best_ms = 1e30f;
  for (const TcLaunchOpts& o : cands) {
    const float ms = b.time([&](cudaStream_t s) { return launch_gemm_tc_opts(c, mode, d, o, s); });
    if (ms < best_ms) {
      best_ms = ms;
      best = o;
    }
  }
  if (best_ms >= 1e30f) return fallback;
  t.store(key, best.split * 4 + best.pair + 1);
  return best;
}

int tuned_fma_tile(DeviceCtx* c, int64_t M, int64_t N, int64_t K, cudaStream_t stream) {
  if (const char* e = std::getenv("GBBLAS_FMA_TILE"); e && e[0] >= '0' && e[0] <= '4') return e[0] - '0';
  Tuner& t = Tuner::get();
  const int bm = log2_bucket(M), bn = log2_bucket(N), bk = log2_bucket(K);
  const std::string key = "gemm_fma_tile|" + device_tag(c) + "|m" + std::to_string(bm) + "|n" + std::to_string(bn) +
                          "|k" + std::to_string(bk) + "|f32";
  const int v = t.lookup(key);
  if (v >= 0) return v;
  if (!t.enabled() || capturing(stream) || (double)M * N * K < 1.0e8) return -1;  // small: the tile-count rule
  int64_t m, n, k;
  bucket_shape(bm, bn, bk, m, n, k);
  GemmBench b(c, m, n, k);
  if (!b.ok()) return -1;
  const gbblas_gemm_desc d = b.desc();
  // 0 = 64 x 64, 1 = 128 x 128 (register-staged), 2 = TMA-fed 128 x 128,
  // 3 = TMA-fed stream-K, offered where whole tiles fill the SMs badly, 4 =
  // TMA-fed cluster pairs, offered where two CTAs per tile fill the SMs in
  // one wave (the TMA kernels' eligibility is the caller's operands': an
  // ineligible call falls back)
  std::vector<int> tiles{0, 1, 2};
  if (sgemm_tma_streamk_useful(c, m, n, k)) tiles.push_back(3);
  if (sgemm_tma_pairs_useful(c, m, n, k)) tiles.push_back(4);
  int best = -1;
  float best_ms = 1e30f;
  for (int tile : tiles) {
    const float ms = b.time([&](cudaStream_t s) {
      return launch_gemm_fma<float>(c, d.M, d.N, d.K, d.A, d.rsa, d.csa, d.B, d.rsb, d.csb, d.C, d.rsc, d.csc, s, 0,
                                    tile);
    });
    if (ms < best_ms) {
      best_ms = ms;
      best = tile;
    }
  }
  if (best < 0) return -1;
  t.store(key, best);
  return best;
}

}  // namespace gbblas
