// Errors, allocation, timing and kernel profiling shared by the library.
#include <chrono>
#include <cstdarg>
#include <cstring>
#include <map>
#include <mutex>
#include <string>

#include "la3g_internal.h"

namespace la3g {

static thread_local int tls_code = LA3G_OK;
static thread_local char tls_msg[1024] = "";
thread_local uint32_t tls_launches = 0;

int set_error(int code, const char* fmt, ...)
{
  tls_code = code;
  va_list ap;
  va_start(ap, fmt);
  std::vsnprintf(tls_msg, sizeof tls_msg, fmt, ap);
  va_end(ap);
  return code;
}

int num_sms()
{
  static int cached[64] = {};
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64)
  {
    cudaGetLastError();
    return 152;
  }
  if (!cached[dev])
  {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
    {
      cudaGetLastError();
      v = 152;
    }
    cached[dev] = v;  // the same value from any thread: a benign race
  }
  return cached[dev];
}

double now_ms()
{
  using namespace std::chrono;
  return duration<double, std::milli>(steady_clock::now().time_since_epoch()).count();
}

int galloc_bytes(la3g_graph* G, void** p, size_t bytes)
{
  *p = nullptr;
  cudaError_t e = cudaMalloc(p, bytes ? bytes : 16);
  if (e != cudaSuccess)
  {
    cudaGetLastError();
    *p = nullptr;
    return set_error(LA3G_ENOMEM, "device allocation of %zu bytes failed: %s", bytes, cudaGetErrorString(e));
  }
  G->allocations.push_back(*p);
  G->device_bytes += bytes;
  return LA3G_OK;
}

// ---------------------------------------------------------------- profiling

namespace {
struct KStat
{
  uint64_t launches = 0;
  double ms = 0, bytes = 0;
};
std::mutex prof_mu;
std::map<std::string, KStat> prof_table;
bool prof_on = false;
}  // namespace

ProfileScope::ProfileScope(const char* name_, cudaStream_t s, double bytes_)
    : name(name_), stream(s), bytes(bytes_)
{
  tls_launches++;
  if (!prof_on) return;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
  {
    cudaGetLastError();
    e0 = e1 = nullptr;
    return;
  }
  cudaEventRecord(e0, stream);
}

ProfileScope::~ProfileScope()
{
  if (!e0) return;
  cudaEventRecord(e1, stream);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  std::lock_guard<std::mutex> lock(prof_mu);
  KStat& k = prof_table[name];
  k.launches++;
  k.ms += ms;
  k.bytes += bytes;
}

bool profile_enabled() { return prof_on; }

DeviceLoop::~DeviceLoop()
{
  if (exec) cudaGraphExecDestroy(exec);
}

void profile_add_bytes(const char* name, double bytes)
{
  if (!prof_on) return;
  std::lock_guard<std::mutex> lock(prof_mu);
  prof_table[name].bytes += bytes;
}

CallTimer::CallTimer(la3g_graph* G_, la3g_stats* st_) : G(G_), st(st_), t0(now_ms()), launches0(tls_launches)
{
  if (st) std::memset(st, 0, sizeof *st);
}

void CallTimer::device_begin() { cudaEventRecord(G->ev0, G->stream); }
void CallTimer::device_end() { cudaEventRecord(G->ev1, G->stream); }

int CallTimer::finish()
{
  LA3G_CUDA(cudaStreamSynchronize(G->stream));
  if (st)
  {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, G->ev0, G->ev1) != cudaSuccess) { cudaGetLastError(); ms = 0; }
    st->device_ms = ms;
    st->host_ms = now_ms() - t0;
    st->kernel_launches = tls_launches - launches0;
  }
  return LA3G_OK;
}

}  // namespace la3g

using namespace la3g;

extern "C" const char* la3g_last_error_string(void) { return tls_msg; }

extern "C" const char* la3g_status_string(int s)
{
  switch (s)
  {
    case LA3G_OK: return "ok";
    case LA3G_EINVAL: return "invalid argument";
    case LA3G_EIO: return "i/o error";
    case LA3G_EFORMAT: return "bad file format";
    case LA3G_ENOMEM: return "out of memory";
    case LA3G_EBUDGET: return "over the HBM budget";
    case LA3G_ETIMEOUT: return "device wait timed out";
    case LA3G_ECUDA: return "CUDA error";
    case LA3G_EBUSY: return "busy";
    default: return "unknown status";
  }
}

extern "C" void la3g_profile_enable(int on)
{
  std::lock_guard<std::mutex> lock(prof_mu);
  prof_on = on != 0;
}

extern "C" void la3g_profile_reset(void)
{
  std::lock_guard<std::mutex> lock(prof_mu);
  prof_table.clear();
}

extern "C" size_t la3g_profile_report(char* buf, size_t cap)
{
  std::lock_guard<std::mutex> lock(prof_mu);
  std::string s = "{";
  bool first = true;
  char tmp[512];
  for (auto& kv : prof_table)
  {
    std::snprintf(tmp, sizeof tmp, "%s\"%s\": {\"launches\": %llu, \"ms\": %.6f, \"bytes\": %.0f}",
                  first ? "" : ", ", kv.first.c_str(), (unsigned long long) kv.second.launches, kv.second.ms,
                  kv.second.bytes);
    s += tmp;
    first = false;
  }
  s += "}";
  if (buf && cap)
  {
    size_t n = s.size() < cap - 1 ? s.size() : cap - 1;
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return s.size();
}
