#include <cstdlib>
#include <cstring>
#include <mutex>

#include "vj_host.h"

namespace vj {
namespace host {

bool gpu_ready()
{
  static int ok = -1;
  if (ok < 0) {
    int cnt = 0;
    ok = ((cudaGetDeviceCount(&cnt) == cudaSuccess) && (cnt > 0)) ? 1 : 0;
  }
  return ok == 1;
}

int device_slot()
{
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0)
    dev = 0;
  return dev & (MAX_DEVICES - 1);
}

int sm_count()
{
  // per device: a process may drive GPUs of different sizes (grids are sized for the
  // current device of each call)
  static int cnt[MAX_DEVICES] = {};
  const int dev = device_slot();
  int &n = cnt[dev];
  if (!n) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0)
      v = 1;
    n = v;
  }
  return n;
}

bool host_pinned(const void *p)
{
  if (!p)
    return true;
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return at.type == cudaMemoryTypeHost;
}

bool pageable_access()
{
  static int vs[MAX_DEVICES] = {};  // 0 unknown, 1 yes, 2 no
  const int dev = device_slot();
  int &v = vs[dev];
  if (!v) {
    int a = 0;
    if (cudaDeviceGetAttribute(&a, cudaDevAttrPageableMemoryAccess, dev) != cudaSuccess)
      a = 0;
    const char *e = getenv("VJ_STAGED");
    if (e && *e == '1')
      a = 0;
    v = a ? 1 : 2;
  }
  return v == 1;
}

bool Staging::reserve(size_t bytes)
{
  if (bytes <= size)
    return true;
  if (ptr) {
    cudaDeviceSynchronize();
    cudaFree(ptr);
    ptr = nullptr;
    size = 0;
  }
  if (cudaMalloc(&ptr, bytes) != cudaSuccess) {
    ptr = nullptr;
    cudaGetLastError();
    return false;
  }
  size = bytes;
  return true;
}

// (each on the current device: one instance per device)
Staging &staging()
{
  static Staging s[MAX_DEVICES];
  return s[device_slot()];
}

unsigned *batch_queue()
{
  static Staging q[MAX_DEVICES];
  Staging &b = q[device_slot()];
  return b.reserve(256) ? reinterpret_cast<unsigned *>(b.ptr) : nullptr;
}

Staging &staging2()
{
  static Staging s[MAX_DEVICES];
  return s[device_slot()];
}

Staging &staging3()
{
  static Staging s[MAX_DEVICES];
  return s[device_slot()];
}

bool streams2(cudaStream_t s[2])
{
  static std::mutex mu;
  static cudaStream_t st[MAX_DEVICES][2] = {};
  static int made[MAX_DEVICES] = {};  // 0 not yet, 1 made, -1 failed
  const int dev = device_slot();
  std::lock_guard<std::mutex> lk(mu);
  if (!made[dev])
    made[dev] = ((cudaStreamCreateWithFlags(&st[dev][0], cudaStreamNonBlocking) == cudaSuccess) &&
                 (cudaStreamCreateWithFlags(&st[dev][1], cudaStreamNonBlocking) == cudaSuccess))
                    ? 1
                    : -1;
  s[0] = st[dev][0];
  s[1] = st[dev][1];
  return made[dev] == 1;
}

std::recursive_mutex &host_call_lock()
{
  static std::recursive_mutex m[MAX_DEVICES];
  return m[device_slot()];
}

long long bjac2_chunk(long long n, size_t elem, bool cplx, int lanes)
{
  // about 512 MiB of device staging per buffer
  const size_t per_elem = elem * (cplx ? 9 : 7) + 1;
  long long c = (long long)((size_t)512 << 20) / (long long)per_elem;
  c -= c % (lanes * 64);
  if (c < lanes * 64)
    c = lanes * 64;
  if (c > n)
    c = n;
  return c;
}

// the calling thread's last call (each host thread keeps its own record)
static thread_local vj_trace g_trace;

void trace_reset()
{
  memset(&g_trace, 0, sizeof(g_trace));
}

bool trace_enabled()
{
  const char *e = getenv("VJ_TRACE");
  return e && *e == '1';
}

void trace_phases(const unsigned long long *cycles, int count)
{
  for (int i = 0; i < count && i < 8; ++i)
    g_trace.phase_cycles[i] = cycles[i];
}

void trace_sweep(unsigned sweep, unsigned long long rotations)
{
  if (sweep < 64)
    g_trace.rotations[sweep] = rotations;
  g_trace.sweeps = sweep + 1;
}

static thread_local double g_mixed[6];

void mixed_phases_set(double fp32, double gemm, double fp64, double fin, double fp32_steps, double block)
{
  g_mixed[0] = fp32;
  g_mixed[1] = gemm;
  g_mixed[2] = fp64;
  g_mixed[3] = fin;
  g_mixed[4] = fp32_steps;
  g_mixed[5] = block;
}

}  // namespace host
}  // namespace vj

extern "C" vj_fint vj_last_mixed_phases(double out[6])
{
  if (!out)
    return VJ_ERR_ARG;
  for (int i = 0; i < 6; ++i)
    out[i] = vj::host::g_mixed[i];
  return 0;
}

extern "C" vj_fint vj_last_trace(vj_trace *out)
{
  if (!out)
    return VJ_ERR_ARG;
  *out = vj::host::g_trace;
  return 0;
}

extern "C" int vj_abi_int_bits(void) { return (int)(8 * sizeof(vj_fint)); }

extern "C" const char *vj_version(void)
{
  return "vecjac_gb300 0.1 (sm_103a)";
}
