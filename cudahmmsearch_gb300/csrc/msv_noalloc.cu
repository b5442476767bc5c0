// msv_noalloc.cu -- a search entry point that allocates no device memory.
//
// Who needs it: callers that must not call cudaMalloc while searching, such
// as a serving process whose device memory is entirely owned by another
// allocator (a framework that reserves the whole GPU up front), or a real-time
// loop that forbids allocation after start-up because cudaMalloc can
// synchronise the device and fail under memory pressure. They create the
// profile and database once, at set-up, and from then on call
// msvgb_search_static() with output buffers they already own.
//
// msvgb_search() needs, besides its inputs and outputs, a work ticket and two
// per-length tables (tjb_b and the smallest passing xJ) that it allocates on
// first use. Here those live in one file-scope __device__ array instead, so
// the call itself allocates nothing: it fills the array and launches the same
// kernel.
#include <cstring>
#include <mutex>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"

using namespace msvgb;
using namespace msvgb_detail;

namespace {

// Layout of the scratch array: [0, 8) work ticket (must start at zero every
// call); [256, 256 + MAXLEN + 1) tjb_b per length; then, 256-aligned, the
// smallest passing xJ per length.
constexpr size_t kTicketBytes = 256;
constexpr size_t kTableBytes = ((size_t) MSVGB_STATIC_MAX_LEN + 1 + 255) / 256 * 256;
constexpr size_t kScratchBytes = kTicketBytes + 2 * kTableBytes;

// Every GPU that loads this library holds these bytes (about 129 KiB) until
// the process exits.
static __device__ __align__(256) uint8_t g_static_scratch[kScratchBytes];

constexpr int kMaxDevices = 64;
std::mutex g_setup_mu;
uint8_t *g_scratch_addr[kMaxDevices] = {};   // device address of g_static_scratch, per device

// Once per device, with that device current: the device address of the
// array. (Host code cannot use g_static_scratch's own name as an address.)
// The address is kept for the life of the process: it does not survive a
// reset of the device's primary context (cudaDeviceReset), after which this
// entry point must not be called again in the same process.
int scratch_address(int device, uint8_t **out) {
  if (device < 0 || device >= kMaxDevices) return fail(MSVGB_eslEINVAL, "device index out of range");
  std::lock_guard<std::mutex> lock(g_setup_mu);
  if (!g_scratch_addr[device]) {
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_static_scratch);
    if (e != cudaSuccess)
      return fail(MSVGB_eslESYS, std::string("cudaGetSymbolAddress(static scratch): ") + cudaGetErrorString(e));
    g_scratch_addr[device] = (uint8_t *) p;
  }
  *out = g_scratch_addr[device];
  return MSVGB_eslOK;
}

struct DeviceGuard {   // restores the caller's current device
  int old = -1;
  DeviceGuard() { cudaGetDevice(&old); }
  ~DeviceGuard() { if (old >= 0) cudaSetDevice(old); }
};

}  // namespace

extern "C" int msvgb_search_static(const msvgb_profile *p, const msvgb_db *db, double F1,
                                   void *d_xj, void *d_flags, void *cuda_stream) {
  if (!p || !db) return fail(MSVGB_eslEINVAL, "NULL profile or database");
  if (db->n > 0 && (!d_xj || !d_flags)) return fail(MSVGB_eslEINVAL, "NULL output buffer");
  if (p->ctx != db->ctx) return fail(MSVGB_eslEINVAL, "profile and database belong to different contexts");
  if (db->Lmax > MSVGB_STATIC_MAX_LEN)
    return fail(MSVGB_eslEINVAL, "msvgb_search_static: a sequence is longer than MSVGB_STATIC_MAX_LEN (" +
                                     std::to_string(MSVGB_STATIC_MAX_LEN) + "); use msvgb_search_device");
  if (db->n == 0) return MSVGB_eslOK;

  const msvgb_ctx *c = p->ctx;
  DeviceGuard guard;
  cudaError_t e = cudaSetDevice(c->device);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("cudaSetDevice: ") + cudaGetErrorString(e));
  uint8_t *scratch = nullptr;
  int st = scratch_address(c->device, &scratch);
  if (st != MSVGB_eslOK) return st;

  // Per-length tables on the host (host memory only), exactly as msvgb_search builds them.
  const int Lmax = db->Lmax;
  std::vector<uint8_t> tjb(Lmax + 1), xjm(Lmax + 1, 255);
  for (int L = 0; L <= Lmax; ++L) tjb[L] = msvgb_tjb_b(p->scale, L);
  for (int L : db->distinct_len) {
    if (L == 0) continue;
    const int v = xjmin_for(p, L, F1);
    if (v < 0) return fail(MSVGB_eslESYS, "F1 pass set is not monotone in xJ");
    xjm[L] = (uint8_t) v;
  }

  cudaStream_t s = cuda_stream ? (cudaStream_t) cuda_stream : c->stream;
  if (db->ready) {                                   // a database still being packed, as msvgb_search_device waits
    e = cudaStreamWaitEvent(s, db->ready, 0);
    if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("cudaStreamWaitEvent: ") + cudaGetErrorString(e));
  }
  uint8_t *d_ticket = scratch;
  uint8_t *d_tjb = scratch + kTicketBytes;
  uint8_t *d_xjmin = scratch + kTicketBytes + kTableBytes;
  // The array keeps the previous call's contents: the ticket must restart at
  // zero, and both tables are rewritten over [0, Lmax]. The tables are copied
  // from pageable host memory (this call allocates no pinned buffer): the
  // runtime waits for the stream's earlier work before such a copy and
  // returns once it has taken the bytes, so the vectors may go when it returns.
  e = cudaMemsetAsync(d_ticket, 0, sizeof(unsigned long long), s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_tjb, tjb.data(), Lmax + 1, cudaMemcpyHostToDevice, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_xjmin, xjm.data(), Lmax + 1, cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("static scratch upload: ") + cudaGetErrorString(e));

  // Always the fused 32-lane kernel, whatever lanes the profile was given:
  // the lane-group pass needs a list of undecided sequences as long as the
  // database, which a fixed-size array cannot hold.
  ProfDev P;
  P.M = p->M; P.C = p->C; P.tbm = p->tbm; P.tec = p->tec; P.base = p->base; P.bias = p->bias;
  P.stab = p->d_stab; P.mtab = p->d_mtab; P.tjb = d_tjb; P.xjmin = d_xjmin; P.ssv_f16 = p->f16;
  LaunchArgs a;
  a.P = P;
  a.db = DbDev{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  a.out_xj = (uint8_t *) d_xj; a.out_flags = (uint8_t *) d_flags;
  a.ticket = (unsigned long long *) d_ticket;
  a.stream = s; a.grid = 0; a.skip_empty = 1;
  e = dispatch(p->C, p->f16 != 0, a, c->num_sms);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("msvgb_search_static launch: ") + cudaGetErrorString(e));
  count_launch();
  return MSVGB_eslOK;
}
