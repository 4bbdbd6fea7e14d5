// autotune.cu — launch-shape autotuner.
//
// Some launch shapes of the step have no single best value across grids,
// orbital counts and GPUs: the L2 prefetch distance of the copy plane pass,
// the tile width (lines per CTA) of the z pass, the orbitals per CTA of the
// box-term kernel, the block size of the dense stage pass.  For each such
// launch site (keyed by its shape: extents, batch, operation) the tuner runs
// the candidates in turn on the launches the computation makes anyway,
// kTuneRounds times each, brackets each with CUDA events on the context's
// stream, and from then on launches the fastest.  Every candidate computes
// the same arithmetic in the same order (they differ only in how work is
// grouped into CTAs and what is prefetched), so results are bit-identical
// whatever the tuner picks; sites whose candidates would change a summation
// order (split-K Gram sums, segment sums of the gathers) are not tuned.
// While the stream is being captured into a graph no events are recorded and
// the site's current choice (or its default) is launched.
#include <algorithm>
#include <cstdio>
#include <string>

#include "common.cuh"

namespace opaw {

constexpr int kTuneRounds = 2;

static TuneSite *find_site(opaw_ctx *c, const std::string &key) {
  for (auto &kv : c->tune)
    if (kv.first == key) return &kv.second;
  return nullptr;
}

int tune_begin(opaw_ctx *c, const std::string &key, const std::vector<std::string> &labels, int dflt,
               TuneSite **timed) {
  *timed = nullptr;
  const int n = (int)labels.size();
  if (c->tune_on == 0 || n <= 1) return dflt;
  TuneSite *s = find_site(c, key);
  if (s && s->chosen >= 0) return s->chosen;
  if (c->tune_on == 2) return dflt;  // frozen: no more timing
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(c->stream, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return dflt;
  if (!s) {
    c->tune.emplace_back(key, TuneSite());
    s = &c->tune.back().second;
    s->labels = labels;
    s->ev.assign((size_t)2 * n * kTuneRounds, nullptr);
    for (auto &e : s->ev)
      if (cudaEventCreate(&e) != cudaSuccess) {
        e = nullptr;
        s->chosen = dflt;  // no events: keep the default
        return dflt;
      }
  }
  if (s->next == n * kTuneRounds) {
    // every candidate timed: the fastest of its rounds decides
    if (cudaEventSynchronize(s->ev.back()) != cudaSuccess) {
      s->chosen = dflt;
      return dflt;
    }
    s->ms.assign(n, 1e30f);
    for (int r = 0; r < n * kTuneRounds; r++) {
      float t = 0.f;
      if (cudaEventElapsedTime(&t, s->ev[2 * r], s->ev[2 * r + 1]) == cudaSuccess)
        s->ms[r % n] = std::min(s->ms[r % n], t);
    }
    s->chosen = (int)(std::min_element(s->ms.begin(), s->ms.end()) - s->ms.begin());
    for (auto &e : s->ev)
      if (e) cudaEventDestroy(e);
    s->ev.clear();
    return s->chosen;
  }
  const int cand = s->next % n;
  if (cudaEventRecord(s->ev[2 * s->next], c->stream) != cudaSuccess) return dflt;
  *timed = s;
  return cand;
}

int tune_end(opaw_ctx *c, TuneSite *s) {
  if (!s) return OPAW_OK;
  OPAW_CUDA(cudaEventRecord(s->ev[2 * s->next + 1], c->stream));
  s->next++;
  return OPAW_OK;
}

void tune_free(opaw_ctx *c) {
  for (auto &kv : c->tune)
    for (auto &e : kv.second.ev)
      if (e) cudaEventDestroy(e);
  c->tune.clear();
}

}  // namespace opaw

using namespace opaw;

int opaw_tune_enable(opaw_ctx *c, int mode) {
  OPAW_ARG(c, "null context");
  OPAW_ARG(mode >= 0 && mode <= 2, "mode must be 0 (off), 1 (on) or 2 (frozen)");
  c->tune_on = mode;
  return OPAW_OK;
}

static std::string json_str(const std::string &s) {
  std::string o = "\"";
  for (char ch : s) {
    if (ch == '"' || ch == '\\') o += '\\';
    o += ch;
  }
  return o + "\"";
}

int opaw_tune_report(opaw_ctx *c, char *buf, int64_t len, int64_t *needed) {
  OPAW_ARG(c, "null context");
  std::string o = "[";
  for (size_t i = 0; i < c->tune.size(); i++) {
    const TuneSite &s = c->tune[i].second;
    if (i) o += ", ";
    o += "{\"site\": " + json_str(c->tune[i].first) + ", \"candidates\": [";
    for (size_t j = 0; j < s.labels.size(); j++) o += (j ? ", " : "") + json_str(s.labels[j]);
    o += "], \"ms\": [";
    for (size_t j = 0; j < s.ms.size(); j++) {
      char t[32];
      std::snprintf(t, sizeof(t), "%s%.6g", j ? ", " : "", (double)s.ms[j]);
      o += t;
    }
    o += "], \"chosen\": " + std::to_string(s.chosen) + "}";
  }
  o += "]";
  if (needed) *needed = (int64_t)o.size() + 1;
  if (buf && len > 0) {
    const size_t k = std::min((size_t)len - 1, o.size());
    o.copy(buf, k);
    buf[k] = '\0';
  }
  return OPAW_OK;
}
