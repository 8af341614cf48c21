// Per-operator device timing (see prof.h) and its C entry points.
#include <atomic>
#include <mutex>
#include <vector>
#include "../../include/csem_gpu.h"
#include "prof.h"

namespace csem {

namespace {
struct Rec {
  int cat, units;
  cudaEvent_t a, b;
  bool closed;
};
std::atomic<bool> g_on{false};
std::mutex g_mu;  // records may come from several host threads (one per context)
std::vector<Rec> g_recs;
std::vector<cudaEvent_t> g_pool;

cudaEvent_t get_event()
{
  if (!g_pool.empty()) {
    cudaEvent_t e = g_pool.back();
    g_pool.pop_back();
    return e;
  }
  cudaEvent_t e;
  cudaEventCreate(&e);
  return e;
}
}  // namespace

static std::atomic<long long> g_launches{0};
void count_launch(int n) { g_launches += n; }

bool prof_on() { return g_on; }

int prof_begin(int cat, cudaStream_t st, int units)
{
  std::lock_guard<std::mutex> lock(g_mu);
  Rec r;
  r.cat = cat;
  r.units = units;
  r.a = get_event();
  r.b = get_event();
  r.closed = false;
  cudaEventRecord(r.a, st);
  g_recs.push_back(r);
  return (int)g_recs.size() - 1;
}

void prof_end(int tok, cudaStream_t st)
{
  std::lock_guard<std::mutex> lock(g_mu);
  if (tok < 0 || tok >= (int)g_recs.size()) return;
  cudaEventRecord(g_recs[tok].b, st);
  g_recs[tok].closed = true;
}

}  // namespace csem

extern "C" {

/* Enable (1) or disable (0) per-operator timing; enabling clears earlier records. */
int csem_profile(int enable)
{
  using namespace csem;
  cudaDeviceSynchronize();
  std::lock_guard<std::mutex> lock(g_mu);
  for (auto& r : g_recs) {
    g_pool.push_back(r.a);
    g_pool.push_back(r.b);
  }
  g_recs.clear();
  g_on = enable != 0;
  return CSEM_OK;
}

/* Kernel launches issued by this library since it was loaded. */
long long csem_launch_count(void) { return csem::g_launches; }

/* ms[cat] = summed device milliseconds, count[cat] = applications, units[cat] =
 * systems processed summed over applications; cat < ncat. */
int csem_profile_read(int ncat, double* ms, long* count, long* units)
{
  using namespace csem;
  cudaDeviceSynchronize();
  std::lock_guard<std::mutex> lock(g_mu);
  for (int c = 0; c < ncat; c++) {
    ms[c] = 0;
    count[c] = 0;
    if (units) units[c] = 0;
  }
  for (auto& r : g_recs) {
    if (!r.closed || r.cat >= ncat) continue;
    float t = 0;
    if (cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
      ms[r.cat] += t;
      count[r.cat] += 1;
      if (units) units[r.cat] += r.units;
    }
  }
  return CSEM_OK;
}

}  // extern "C"
