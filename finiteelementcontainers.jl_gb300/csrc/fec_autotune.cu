// fec_autotune.cu -- see fec_autotune.h.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <string>
#include <vector>
#include "../../include/fec_gb300.h"
#include "fec_autotune.h"

namespace fec {
namespace {

struct Entry {
  std::string family;
  int device = 0, bucket = 0, choice = 0;
  std::vector<std::string> labels;
  std::vector<float> ms;
};

std::mutex g_mu;
std::vector<Entry> g_entries;

bool tuning_enabled() {
  const char* v = std::getenv("FEC_AUTOTUNE");
  return !(v && v[0] == '0');
}

// FEC_AUTOTUNE_CANDIDATE=i forces candidate i of every family (where it exists).
int forced_candidate() {
  const char* v = std::getenv("FEC_AUTOTUNE_CANDIDATE");
  return (v && v[0] >= '0' && v[0] <= '9') ? std::atoi(v) : -1;
}

int size_bucket(int64_t ne) {  // factors of 4 in the element count
  int b = 0;
  while (ne >= 4 && b < 30) {
    ne /= 4;
    ++b;
  }
  return b;
}

}  // namespace

cudaError_t tuned_launch(const char* family, const TuneCandidate* cand, int n, int dflt, const ElemArgs& a,
                         cudaStream_t s) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  const int bucket = size_bucket(a.ne);
  const int forced = forced_candidate();
  if (forced >= 0 && forced < n) return cand[forced].fn(a, s);
  if (!tuning_enabled()) return cand[dflt].fn(a, s);
  {
    std::lock_guard<std::mutex> lk(g_mu);
    for (const Entry& en : g_entries)
      if (en.device == dev && en.bucket == bucket && en.family == family) return cand[en.choice].fn(a, s);
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if ((e = cudaStreamIsCapturing(s, &cs)) != cudaSuccess) return e;
  if (cs != cudaStreamCaptureStatusNone || n <= 1) return cand[dflt].fn(a, s);
  Entry en;
  en.family = family;
  en.device = dev;
  en.bucket = bucket;
  cudaEvent_t t0, t1;
  if ((e = cudaEventCreate(&t0)) != cudaSuccess) return e;
  if ((e = cudaEventCreate(&t1)) != cudaSuccess) {
    cudaEventDestroy(t0);
    return e;
  }
  float best = INFINITY;
  for (int i = 0; i < n && e == cudaSuccess; ++i) {
    // one untimed run (attributes, instruction cache), then one timed run
    if ((e = cand[i].fn(a, s)) != cudaSuccess) break;
    if ((e = cudaEventRecord(t0, s)) != cudaSuccess) break;
    if ((e = cand[i].fn(a, s)) != cudaSuccess) break;
    if ((e = cudaEventRecord(t1, s)) != cudaSuccess) break;
    if ((e = cudaEventSynchronize(t1)) != cudaSuccess) break;
    float ms = 0.f;
    if ((e = cudaEventElapsedTime(&ms, t0, t1)) != cudaSuccess) break;
    en.labels.push_back(cand[i].label);
    en.ms.push_back(ms);
    if (ms < best) {
      best = ms;
      en.choice = i;
    }
  }
  cudaEventDestroy(t0);
  cudaEventDestroy(t1);
  if (e != cudaSuccess) return e;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    g_entries.push_back(en);
  }
  // the outputs are those of the last candidate, identical to the chosen one's
  return cudaSuccess;
}

int tuned_report(char* buf, size_t len) {
  std::lock_guard<std::mutex> lk(g_mu);
  std::string out;
  for (const Entry& en : g_entries) {
    char line[512];
    int k = snprintf(line, sizeof line, "%s bucket=%d device=%d choice=%s |", en.family.c_str(), en.bucket, en.device,
                     en.labels.empty() ? "-" : en.labels[en.choice].c_str());
    for (size_t i = 0; i < en.labels.size() && k > 0 && k < int(sizeof line); ++i)
      k += snprintf(line + k, sizeof line - k, " %s %.4f ms;", en.labels[i].c_str(), double(en.ms[i]));
    out += line;
    out += "\n";
  }
  if (buf && len) {
    snprintf(buf, len, "%s", out.c_str());
  }
  return int(g_entries.size());
}

}  // namespace fec

extern "C" int fec_autotune_report(char* buf, size_t len) { return fec::tuned_report(buf, len); }
