// Autotuner of launch shapes.  A tuned parameter is an integer choice among candidates (a contraction tile, a
// gather tile, a scatter column group) for one problem shape; only choices that leave every result bitwise
// unchanged are tuned.  Each candidate is run once to warm up and three times between CUDA events on the
// caller's stream; the fastest mean wins.  Choices
// are kept per (shape, parameter) for the life of the process and in a JSON cache file keyed by the device and
// the library's source build, so a later process on the same device skips the measurement.
//
// Environment:
//   WTB_TUNE_CACHE   path of the cache file; "off" keeps choices in memory only.  Default:
//                    $XDG_CACHE_HOME/wtb_gb300/autotune.json, else $HOME/.cache/wtb_gb300/autotune.json
//   WTB_TUNE=off     no measurement: every parameter takes its default, the rule the caller uses untuned (or
//                    its pin)
//   WTB_TUNE_PIN     "param=value,..." pins parameters without timing (a kernel profiler serialises and replays
//                    the timed runs, so a profiled process would otherwise tune differently from a normal one)
//   WTB_TC_TILE      256 | 128: the pin of the contraction tile (same as WTB_TUNE_PIN=tile_n=...)
//
// Cache format: {"format": "wtb_gb300 autotune 1", "entries": [{"device": ..., "build": ..., "shape": ...,
// "param": ..., "choice": N, "ms": [[candidate, mean ms], ...]}, ...]}.  An entry applies only where device,
// build, shape and parameter all match and its choice is among the caller's candidates.
#include "wtb_internal.h"

#include <sys/stat.h>
#include <unistd.h>

#include <cerrno>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>
#include <string>
#include <vector>

#ifndef WTB_SOURCE_HASH
#define WTB_SOURCE_HASH "unversioned"
#endif

namespace wtb {
namespace {

// ------------------------------------------------------------------------------------------ minimal JSON reader
// Objects, arrays, strings (with the escapes this file writes: \" \\ \/ \n \t \uXXXX below 0x80), numbers,
// true/false/null.  Anything else makes the whole file unusable (the cache is then ignored and rewritten).
struct JVal {
  enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
  double num = 0.0;
  bool b = false;
  std::string str;
  std::vector<JVal> arr;
  std::vector<std::pair<std::string, JVal>> obj;
  const JVal* get(const char* k) const {
    for (const auto& kv : obj)
      if (kv.first == k) return &kv.second;
    return nullptr;
  }
};

struct JParser {
  const std::string& t;
  size_t i = 0;
  int depth = 0;
  explicit JParser(const std::string& text) : t(text) {}
  void ws() {
    while (i < t.size() && (t[i] == ' ' || t[i] == '\n' || t[i] == '\r' || t[i] == '\t')) ++i;
  }
  bool lit(const char* w) {
    const size_t n = std::strlen(w);
    if (t.compare(i, n, w) != 0) return false;
    i += n;
    return true;
  }
  bool string(std::string* out) {
    if (i >= t.size() || t[i] != '"') return false;
    ++i;
    out->clear();
    while (i < t.size() && t[i] != '"') {
      char c = t[i++];
      if (c == '\\') {
        if (i >= t.size()) return false;
        const char e = t[i++];
        switch (e) {
          case '"': c = '"'; break;
          case '\\': c = '\\'; break;
          case '/': c = '/'; break;
          case 'n': c = '\n'; break;
          case 't': c = '\t'; break;
          case 'u': {
            if (i + 4 > t.size()) return false;
            const long v = std::strtol(t.substr(i, 4).c_str(), nullptr, 16);
            if (v <= 0 || v >= 0x80) return false;
            c = (char)v;
            i += 4;
            break;
          }
          default: return false;
        }
      }
      out->push_back(c);
    }
    if (i >= t.size()) return false;
    ++i;
    return true;
  }
  bool value(JVal* v) {
    if (++depth > 32) return false;
    ws();
    bool ok = false;
    if (i >= t.size()) {
      ok = false;
    } else if (t[i] == '{') {
      ++i;
      v->kind = JVal::OBJ;
      ws();
      if (i < t.size() && t[i] == '}') {
        ++i;
        ok = true;
      } else {
        while (true) {
          ws();
          std::string k;
          JVal x;
          if (!string(&k)) break;
          ws();
          if (i >= t.size() || t[i] != ':') break;
          ++i;
          if (!value(&x)) break;
          v->obj.emplace_back(std::move(k), std::move(x));
          ws();
          if (i < t.size() && t[i] == ',') {
            ++i;
            continue;
          }
          if (i < t.size() && t[i] == '}') {
            ++i;
            ok = true;
          }
          break;
        }
      }
    } else if (t[i] == '[') {
      ++i;
      v->kind = JVal::ARR;
      ws();
      if (i < t.size() && t[i] == ']') {
        ++i;
        ok = true;
      } else {
        while (true) {
          JVal x;
          if (!value(&x)) break;
          v->arr.push_back(std::move(x));
          ws();
          if (i < t.size() && t[i] == ',') {
            ++i;
            continue;
          }
          if (i < t.size() && t[i] == ']') {
            ++i;
            ok = true;
          }
          break;
        }
      }
    } else if (t[i] == '"') {
      v->kind = JVal::STR;
      ok = string(&v->str);
    } else if (lit("true")) {
      v->kind = JVal::BOOL;
      v->b = ok = true;
    } else if (lit("false")) {
      v->kind = JVal::BOOL;
      ok = true;
    } else if (lit("null")) {
      ok = true;
    } else {
      const char* p0 = t.c_str() + i;
      char* p1 = nullptr;
      errno = 0;
      v->num = std::strtod(p0, &p1);
      v->kind = JVal::NUM;
      ok = p1 != p0 && errno == 0;
      i += (size_t)(p1 - p0);
    }
    --depth;
    return ok;
  }
};

std::string jstr(const std::string& s) {
  std::string o = "\"";
  for (const char c : s) {
    if (c == '"' || c == '\\') {
      o.push_back('\\');
      o.push_back(c);
    } else if (c == '\n') {
      o += "\\n";
    } else if (c == '\t') {
      o += "\\t";
    } else if ((unsigned char)c < 0x20) {
      char b[8];
      std::snprintf(b, sizeof(b), "\\u%04x", (unsigned)c);
      o += b;
    } else {
      o.push_back(c);
    }
  }
  return o + "\"";
}

// ------------------------------------------------------------------------------------------------- tuner state
struct Choice {
  std::string shape, param, source;  // source: measured | cache | pinned | default
  int choice = 0;
  std::vector<std::pair<int, double>> ms;  // candidate, mean ms (measured or from the cache)
};

struct CacheEntry {
  std::string device, build, shape, param;
  int choice = 0;
  std::vector<std::pair<int, double>> ms;
};

std::mutex g_mu;
std::map<std::string, Choice> g_choices;  // shape + '\n' + param
bool g_loaded = false;
std::vector<CacheEntry> g_file;           // every entry of the cache file (other devices and builds included)

const char* kFormat = "wtb_gb300 autotune 1";

std::string cache_path() {
  const char* p = std::getenv("WTB_TUNE_CACHE");
  if (p) return std::strcmp(p, "off") == 0 ? std::string() : std::string(p);
  if (const char* x = std::getenv("XDG_CACHE_HOME"))
    if (*x) return std::string(x) + "/wtb_gb300/autotune.json";
  if (const char* h = std::getenv("HOME"))
    if (*h) return std::string(h) + "/.cache/wtb_gb300/autotune.json";
  return std::string();
}

std::string device_id() {
  int dev = 0;
  cudaDeviceProp pr;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaGetDeviceProperties(&pr, dev) != cudaSuccess) return "unknown";
  char b[320];
  std::snprintf(b, sizeof(b), "%s sm_%d%d %d SMs", pr.name, pr.major, pr.minor, pr.multiProcessorCount);
  return b;
}

void load_cache_locked() {
  if (g_loaded) return;
  g_loaded = true;
  const std::string path = cache_path();
  if (path.empty()) return;
  std::ifstream f(path);
  if (!f) return;
  std::stringstream ss;
  ss << f.rdbuf();
  const std::string text = ss.str();
  JParser P(text);
  JVal root;
  if (!P.value(&root) || root.kind != JVal::OBJ) return;
  const JVal* fmt = root.get("format");
  const JVal* ent = root.get("entries");
  if (!fmt || fmt->kind != JVal::STR || fmt->str != kFormat || !ent || ent->kind != JVal::ARR) return;
  for (const JVal& e : ent->arr) {
    if (e.kind != JVal::OBJ) continue;
    const JVal *d = e.get("device"), *b = e.get("build"), *s = e.get("shape"), *p = e.get("param"),
               *c = e.get("choice"), *m = e.get("ms");
    if (!d || !b || !s || !p || !c || d->kind != JVal::STR || b->kind != JVal::STR || s->kind != JVal::STR ||
        p->kind != JVal::STR || c->kind != JVal::NUM)
      continue;
    CacheEntry ce{d->str, b->str, s->str, p->str, (int)c->num, {}};
    if (m && m->kind == JVal::ARR)
      for (const JVal& pr : m->arr)
        if (pr.kind == JVal::ARR && pr.arr.size() == 2 && pr.arr[0].kind == JVal::NUM && pr.arr[1].kind == JVal::NUM)
          ce.ms.emplace_back((int)pr.arr[0].num, pr.arr[1].num);
    g_file.push_back(std::move(ce));
  }
}

// rewrites the whole file (write to a temporary beside it, then rename: readers never see a partial file)
void save_cache_locked() {
  const std::string path = cache_path();
  if (path.empty()) return;
  // create the parent directories (one level per '/'), ignoring those that exist
  for (size_t k = 1; k < path.size(); ++k)
    if (path[k] == '/') mkdir(path.substr(0, k).c_str(), 0755);
  std::string o = "{\"format\": " + jstr(kFormat) + ", \"entries\": [";
  for (size_t k = 0; k < g_file.size(); ++k) {
    const CacheEntry& e = g_file[k];
    o += k ? ",\n  " : "\n  ";
    o += "{\"device\": " + jstr(e.device) + ", \"build\": " + jstr(e.build) + ", \"shape\": " + jstr(e.shape) +
         ", \"param\": " + jstr(e.param) + ", \"choice\": " + std::to_string(e.choice) + ", \"ms\": [";
    for (size_t q = 0; q < e.ms.size(); ++q) {
      char b[64];
      std::snprintf(b, sizeof(b), "%s[%d, %.5f]", q ? ", " : "", e.ms[q].first, e.ms[q].second);
      o += b;
    }
    o += "]}";
  }
  o += "\n]}\n";
  const std::string tmp = path + ".tmp" + std::to_string((long)getpid());
  {
    std::ofstream f(tmp, std::ios::trunc);
    if (!f) return;
    f << o;
    if (!f) return;
  }
  if (std::rename(tmp.c_str(), path.c_str()) != 0) std::remove(tmp.c_str());
}

bool pinned(const char* param, int* value) {
  if (std::strcmp(param, "tile_n") == 0)
    if (const char* t = std::getenv("WTB_TC_TILE")) {
      *value = std::atoi(t);
      return true;
    }
  const char* pin = std::getenv("WTB_TUNE_PIN");
  if (!pin) return false;
  const std::string s(pin), key = std::string(param) + "=";
  size_t k = 0;
  while (k < s.size()) {
    size_t e = s.find(',', k);
    if (e == std::string::npos) e = s.size();
    if (s.compare(k, key.size(), key) == 0) {
      *value = std::atoi(s.substr(k + key.size(), e - k - key.size()).c_str());
      return true;
    }
    k = e + 1;
  }
  return false;
}

bool contains(const std::vector<int>& v, int x) {
  for (int y : v)
    if (y == x) return true;
  return false;
}

}  // namespace

int tune_choice(const std::string& shape, const char* param, const std::vector<int>& cands, int dflt,
                const std::function<cudaError_t(int)>& run, cudaStream_t s) {
  if (cands.empty()) return dflt;
  const std::string key = shape + "\n" + param;
  {
    std::lock_guard<std::mutex> lk(g_mu);
    auto it = g_choices.find(key);
    if (it != g_choices.end() && contains(cands, it->second.choice)) return it->second.choice;
  }
  int pin = 0;
  if (pinned(param, &pin)) {
    const int v = contains(cands, pin) ? pin : dflt;
    std::lock_guard<std::mutex> lk(g_mu);
    g_choices[key] = Choice{shape, param, "pinned", v, {}};
    return v;
  }
  cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
  if (cudaStreamIsCapturing(s, &cs) != cudaSuccess || cs != cudaStreamCaptureStatusNone) return dflt;
  const char* off = std::getenv("WTB_TUNE");
  if (cands.size() == 1 || (off && std::strcmp(off, "off") == 0)) {
    const int v = cands.size() == 1 ? cands[0] : dflt;
    std::lock_guard<std::mutex> lk(g_mu);
    g_choices[key] = Choice{shape, param, "default", v, {}};
    return v;
  }
  const std::string dev = device_id();
  {
    std::lock_guard<std::mutex> lk(g_mu);
    load_cache_locked();
    for (const CacheEntry& e : g_file)
      if (e.device == dev && e.build == WTB_SOURCE_HASH && e.shape == shape && e.param == param &&
          contains(cands, e.choice)) {
        g_choices[key] = Choice{shape, param, "cache", e.choice, e.ms};
        return e.choice;
      }
  }
  std::vector<std::pair<int, double>> ms;
  cudaEvent_t a = nullptr, b = nullptr;
  if (cudaEventCreate(&a) != cudaSuccess || cudaEventCreate(&b) != cudaSuccess) {
    if (a) cudaEventDestroy(a);
    return dflt;
  }
  int best = dflt;
  double best_ms = 1e30;
  for (const int c : cands) {
    if (run(c) != cudaSuccess) continue;
    if (cudaEventRecord(a, s) != cudaSuccess) continue;
    bool ok = true;
    for (int r = 0; r < 3 && ok; ++r) ok = run(c) == cudaSuccess;
    float t = 0.f;
    if (ok && cudaEventRecord(b, s) == cudaSuccess && cudaEventSynchronize(b) == cudaSuccess &&
        cudaEventElapsedTime(&t, a, b) == cudaSuccess) {
      ms.emplace_back(c, t / 3.0);
      if (t / 3.0 < best_ms) {
        best_ms = t / 3.0;
        best = c;
      }
    }
  }
  cudaEventDestroy(a);
  cudaEventDestroy(b);
  // a candidate whose launch was refused (e.g. too much shared memory) leaves its error pending: clear it, so
  // that the caller's next check sees its own launches only
  (void)cudaGetLastError();
  std::lock_guard<std::mutex> lk(g_mu);
  g_choices[key] = Choice{shape, param, "measured", best, ms};
  if (!ms.empty()) {
    load_cache_locked();
    bool found = false;
    for (CacheEntry& e : g_file)
      if (e.device == dev && e.build == WTB_SOURCE_HASH && e.shape == shape && e.param == param) {
        e.choice = best;
        e.ms = ms;
        found = true;
      }
    if (!found) g_file.push_back(CacheEntry{dev, WTB_SOURCE_HASH, shape, param, best, ms});
    save_cache_locked();
  }
  return best;
}

std::string tune_report() {
  const std::string path = cache_path();
  std::lock_guard<std::mutex> lk(g_mu);
  std::string o = "{\"build\": " + jstr(WTB_SOURCE_HASH) + ", \"cache\": " + (path.empty() ? "null" : jstr(path)) +
                  ", \"choices\": [";
  bool first = true;
  for (const auto& kv : g_choices) {
    const Choice& c = kv.second;
    o += first ? "" : ", ";
    first = false;
    o += "{\"shape\": " + jstr(c.shape) + ", \"param\": " + jstr(c.param) + ", \"choice\": " +
         std::to_string(c.choice) + ", \"source\": " + jstr(c.source) + ", \"ms\": [";
    for (size_t q = 0; q < c.ms.size(); ++q) {
      char b[64];
      std::snprintf(b, sizeof(b), "%s[%d, %.5f]", q ? ", " : "", c.ms[q].first, c.ms[q].second);
      o += b;
    }
    o += "]}";
  }
  return o + "]}";
}

std::string tune_cache_path() { return cache_path(); }

}  // namespace wtb
