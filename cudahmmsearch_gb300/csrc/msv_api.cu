// msv_api.cu -- host side of the C ABI in include/msvgb.h.
//
// Owns the device-resident profile layout (the GB300 replacement of the fork's
// loadOM, code/src/GPUFunction.cu:260-294), the packed length-sorted database
// (replacing loadDBQuad/loadCUDA, GPUFunction.cu:219-255, 332-415, and the
// offline dbsort.c/hmmsort.cpp length sort), the per-length tables that keep
// every floating-point expression on the host, and the launches.
//
// Host floating point must round exactly like the reference's x86 build, so
// this file is compiled with -ffp-contract=off (no fused multiply-add).
#include <algorithm>
#include <map>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <unordered_map>
#include <vector>

#include <cuda_fp16.h>
#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_device.cuh"
#include "msv_kernel_impl.cuh"
#include "msv_internal.h"

using namespace msvgb;
using namespace msvgb_detail;

namespace msvgb {
template <int C, bool F16> cudaError_t launch_search(const LaunchArgs &a, int num_sms);
}

// ------------------------------------------------------------------------------
// errors
static thread_local std::string g_err;
static std::atomic<uint64_t> g_launches{0};

namespace msvgb_detail {
int fail(int code, const std::string &msg) { g_err = msg; return code; }
}  // namespace msvgb_detail

extern "C" const char *msvgb_last_error(void) { return g_err.c_str(); }
extern "C" uint64_t msvgb_kernel_launches(void) { return g_launches.load(); }
void msvgb_detail::count_launch() { g_launches.fetch_add(1); }

// ------------------------------------------------------------------------------
// exact host arithmetic of the reference

// unbiased_byteify(logf(3/(L+3))): src/impl_sse/p7_oprofile.c:511-519, 920-925
extern "C" uint8_t msvgb_tjb_b(float scale_b, int L) {
  float sc = logf(3.0f / (float) (L + 3));
  sc = -1.0f * roundf(scale_b * sc);
  return (sc > 255.) ? 255 : (uint8_t) sc;
}

// msvfilter.c:205-210
static float score_from_xj(int xj, int tjb, int base, float scale) {
  float sc = ((float) (xj - tjb) - (float) base);
  sc /= scale;
  sc -= 3.0;
  return sc;
}

extern "C" float msvgb_score(uint8_t xj, uint8_t flags, int L, uint8_t base_b, float scale_b) {
  if (flags & MSVGB_FLAG_ERANGE) return INFINITY;
  return score_from_xj(xj, msvgb_tjb_b(scale_b, L), base_b, scale_b);
}

// p7_bg_SetLength/p7_bg_NullOne (src/p7_bg.c:191-199, 359-363), seq_score and
// the F1 test of p7_Pipeline (src/p7_pipeline.c:673-676), esl_gumbel_surv
// (easel/esl_gumbel.c:129-137).
extern "C" int msvgb_f1_pass(float usc, int L, float mmu, float mlambda, double F1, double *ret_P) {
  // C semantics: log() of a float argument is computed in double (C++'s
  // float overload of log would round differently).
  float p1 = (float) L / (float) (L + 1);
  float nullsc = (float) ((double) (float) L * ::log((double) p1) + ::log(1. - (double) p1));
  float seq_score = (usc - nullsc) / 0.69314718055994529;
  double y = (double) mlambda * ((double) seq_score - (double) mmu);
  double ey = -exp(-y);
  double P = (fabs(ey) < 5e-9) ? -ey : 1 - exp(ey);
  if (ret_P) *ret_P = P;
  return (P > F1) ? 0 : 1;
}

// ------------------------------------------------------------------------------
// objects

static std::atomic<uint64_t> g_db_serial{1};
uint64_t msvgb_detail::next_db_serial() { return g_db_serial.fetch_add(1); }

// DP widths (32-bit words per lane; the warp spans 64*C nodes). f16 tables:
// every C up to 32. int8 tables: even C (two DP words per table word).
static const int kI8C[] = {2, 4, 6, 8, 10, 12, 14, 16, 18, 20, 22, 24, 26, 28, 30, 32, 34, 36, 40, 44, 48, 50};
static const int kF16C[] = {1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 11, 12, 13, 14, 15, 16, 17, 18, 19, 20, 21, 22,
                            23, 24, 25, 26, 27, 28, 29, 30, 31, 32, 34, 36, 38, 40,
                            44, 48, 52, 56, 60, 64, 72, 80, 88, 96, 112, 128};   // above 40: tables in global memory
static const int kMaxF16C = 128;

// Smallest C whose warp spans more than M nodes: node 64*C must be padding
// (the kernels rely on it for the begin value of node 1).
static int need_C(int M) { return M / 64 + 1; }

static int choose_C(int M, bool f16) {
  const int need = need_C(M);
  if (f16) { for (int c : kF16C) if (c >= need) return c; return -1; }
  for (int c : kI8C) if (c >= need) return c;
  return -1;
}

cudaError_t msvgb_detail::dispatch(int C, bool f16, const LaunchArgs &a, int sms) {
#define CASE_I8(c)  case c: return launch_search<c, false>(a, sms);
#define CASE_F16(c) case c: return launch_search<c, true>(a, sms);
  if (f16) {
    switch (C) {
      CASE_F16(1) CASE_F16(2) CASE_F16(3) CASE_F16(4) CASE_F16(5) CASE_F16(6) CASE_F16(7) CASE_F16(8)
      CASE_F16(9) CASE_F16(10) CASE_F16(11) CASE_F16(12) CASE_F16(13) CASE_F16(14) CASE_F16(15) CASE_F16(16)
      CASE_F16(17) CASE_F16(18) CASE_F16(19) CASE_F16(20) CASE_F16(21) CASE_F16(22) CASE_F16(23) CASE_F16(24)
      CASE_F16(25) CASE_F16(26) CASE_F16(27) CASE_F16(28) CASE_F16(29) CASE_F16(30) CASE_F16(31) CASE_F16(32)
      CASE_F16(34) CASE_F16(36) CASE_F16(38) CASE_F16(40)
      CASE_F16(44) CASE_F16(48) CASE_F16(52) CASE_F16(56) CASE_F16(60) CASE_F16(64)
      CASE_F16(72) CASE_F16(80) CASE_F16(88) CASE_F16(96) CASE_F16(112) CASE_F16(128)
    }
  } else {
    switch (C) {
      CASE_I8(2) CASE_I8(4) CASE_I8(6) CASE_I8(8) CASE_I8(10) CASE_I8(12) CASE_I8(14) CASE_I8(16)
      CASE_I8(18) CASE_I8(20) CASE_I8(22) CASE_I8(24) CASE_I8(26) CASE_I8(28) CASE_I8(30) CASE_I8(32)
      CASE_I8(34) CASE_I8(36) CASE_I8(40) CASE_I8(44) CASE_I8(48) CASE_I8(50)
    }
  }
  return cudaErrorInvalidValue;
#undef CASE_I8
#undef CASE_F16
}

namespace msvgb {
template <int C, int G, int CI> cudaError_t launch_ssv_group(const GroupArgs &a, int num_sms);
}

// Mixed-width instantiations (inst_hyb*.cu): (C, G, CI) triples.
#include "msv_hyb_list.h"

// Default 8-bit words per lane of the G-lane SSV pass at DP width C, from a
// sweep on GB300 (1,000,000 sequences; M from 120 to 1008): at 8 lanes none
// below 10 words (4 lost 2.5% at M = 120), 4 up to 17 words (+4 to +7%), 8
// from 18 words (+7 to +10%; 12 and 16 were slower than 8 everywhere); at 16
// lanes 4 up to 23 words (+3 to +9%), 8 from 24 (+8%).
int msvgb_detail::hyb_default_words(int C, int G) {
  if (G == 8) return C < 10 ? 0 : C < 18 ? 4 : 8;
  if (G == 16) return C < 13 ? 0 : C < 24 ? 4 : 8;
  if (G == 32) return C < 17 ? 0 : 8;     // the split 32-lane passes (M 1024-2047): always mixed width
  return 0;
}

bool msvgb_detail::hyb_compiled(int C, int G, int CI) {
#define MSVGB_HYB_HAS(c, g, ci) if (C == c && G == g && CI == ci) return true;
  MSVGB_HYB_LIST(MSVGB_HYB_HAS)
#undef MSVGB_HYB_HAS
  return false;
}

cudaError_t msvgb_detail::dispatch_group(int C, int G, int CI, const GroupArgs &a, int sms) {
  if (CI > 0) {
#define MSVGB_HYB_CALL(c, g, ci) if (C == c && G == g && CI == ci) return launch_ssv_group<c, g, ci>(a, sms);
    MSVGB_HYB_LIST(MSVGB_HYB_CALL)
#undef MSVGB_HYB_CALL
    return cudaErrorInvalidValue;
  }
#define G16(c) case c: return launch_ssv_group<c, 16, 0>(a, sms);
#define G8(c)  case c: return launch_ssv_group<c, 8, 0>(a, sms);
  if (G == 16) {
    switch (C) { G16(2) G16(3) G16(4) G16(5) G16(6) G16(7) G16(8) G16(9) G16(10) G16(11) G16(12) G16(13)
                 G16(14) G16(15) G16(16) G16(17) G16(18) G16(19) G16(20) G16(21) G16(22) G16(23) G16(24)
                 G16(25) G16(26) G16(27) G16(28) G16(29) G16(30) G16(31) G16(32) }
  } else if (G == 8) {
    switch (C) { G8(2) G8(3) G8(4) G8(5) G8(6) G8(7) G8(8) G8(9) G8(10) G8(11) G8(12) G8(13)
                 G8(14) G8(15) G8(16) G8(17) G8(18) G8(19) G8(20) G8(21) G8(22) G8(23) G8(24)
                 G8(25) G8(26) G8(27) G8(28) G8(29) G8(30) G8(31) G8(32) }
  }
  return cudaErrorInvalidValue;
#undef G16
#undef G8
}

namespace msvgb {
template <int C, int G>
cudaError_t launch_list_group(const ProfDev &P, const DbDev &db, uint8_t *out_xj, uint8_t *out_flags,
                              unsigned long long *ticket, const int64_t *list, const unsigned long long *list_count,
                              int num_sms, cudaStream_t stream);
}

cudaError_t msvgb_detail::dispatch_list_group(int C, int G, const ProfDev &P, const DbDev &db, uint8_t *out_xj,
                                              uint8_t *out_flags, unsigned long long *ticket, const int64_t *list,
                                              const unsigned long long *list_count, int sms, cudaStream_t stream) {
#define L32(c) case c: return launch_list_group<c, 32>(P, db, out_xj, out_flags, ticket, list, list_count, sms, stream);
  if (G == 32) {
    switch (C) { L32(17) L32(18) L32(19) L32(20) L32(21) L32(22) L32(23) L32(24) L32(25) L32(26) L32(27)
                 L32(28) L32(29) L32(30) L32(31) L32(32) }
    return cudaErrorInvalidValue;
  }
#undef L32
#define L16(c) case c: return launch_list_group<c, 16>(P, db, out_xj, out_flags, ticket, list, list_count, sms, stream);
#define L8(c)  case c: return launch_list_group<c, 8>(P, db, out_xj, out_flags, ticket, list, list_count, sms, stream);
  if (G == 16) {
    switch (C) { L16(2) L16(3) L16(4) L16(5) L16(6) L16(7) L16(8) L16(9) L16(10) L16(11) L16(12) L16(13)
                 L16(14) L16(15) L16(16) L16(17) L16(18) L16(19) L16(20) L16(21) L16(22) L16(23) L16(24)
                 L16(25) L16(26) L16(27) L16(28) L16(29) L16(30) L16(31) L16(32) }
  } else if (G == 8) {
    switch (C) { L8(2) L8(3) L8(4) L8(5) L8(6) L8(7) L8(8) L8(9) L8(10) L8(11) L8(12) L8(13)
                 L8(14) L8(15) L8(16) L8(17) L8(18) L8(19) L8(20) L8(21) L8(22) L8(23) L8(24)
                 L8(25) L8(26) L8(27) L8(28) L8(29) L8(30) L8(31) L8(32) }
  }
  return cudaErrorInvalidValue;
#undef L16
#undef L8
}

// ------------------------------------------------------------------------------
// context

extern "C" int msvgb_ctx_create(int device, msvgb_ctx **ret_ctx) {
  if (!ret_ctx) return fail(MSVGB_eslEINVAL, "ret_ctx is NULL");
  *ret_ctx = nullptr;
  int ndev = 0;
  CUDA_TRY(cudaGetDeviceCount(&ndev));
  if (device < 0 || device >= ndev) return fail(MSVGB_eslEINVAL, "no such CUDA device");
  CUDA_TRY(cudaSetDevice(device));
  msvgb_ctx *c = new msvgb_ctx();
  c->device = device;
  cudaError_t e = cudaDeviceGetAttribute(&c->num_sms, cudaDevAttrMultiProcessorCount, device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->own, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_ticket, sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaMalloc(&c->d_out, 64);
  if (e == cudaSuccess) e = cudaMalloc(&c->d_bad, sizeof(int));
  if (e == cudaSuccess) e = cudaMalloc(&c->d_aux, 4 * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->side, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->upload, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->dma, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_fork, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventCreateWithFlags(&c->ev_join, cudaEventDisableTiming);
  if (e != cudaSuccess) {
    msvgb_ctx_destroy(c);
    return fail(MSVGB_eslESYS, std::string("context setup: ") + cudaGetErrorString(e));
  }
  c->stream = c->own;
  // MSVGB_TEST_HASH_BITS=b keeps only b bits of the drop-in cache's content
  // hash, so tests can make different profiles collide on purpose.
  if (const char *hb = getenv("MSVGB_TEST_HASH_BITS")) {
    const int b = atoi(hb);
    c->hash_mask = b <= 0 ? 0ull : b >= 64 ? ~0ull : ((1ull << b) - 1ull);
  }
  *ret_ctx = c;
  return MSVGB_eslOK;
}

extern "C" int msvgb_ctx_destroy(msvgb_ctx *c) {
  if (!c) return MSVGB_eslOK;
  cudaSetDevice(c->device);
  for (auto &e : c->dropin) msvgb_profile_destroy(e.p);
  c->dropin.clear();
  if (c->own) cudaStreamSynchronize(c->own);
  cudaFree(c->d_ticket); cudaFree(c->d_out);
  cudaFree(c->d_one); cudaFree(c->d_bad); cudaFree(c->d_aux); cudaFree(c->d_list);
  if (c->own) cudaStreamDestroy(c->own);
  if (c->side) { cudaStreamSynchronize(c->side); cudaStreamDestroy(c->side); }
  if (c->upload) { cudaStreamSynchronize(c->upload); cudaStreamDestroy(c->upload); }
  if (c->dma) { cudaStreamSynchronize(c->dma); cudaStreamDestroy(c->dma); }
  if (c->ev_fork) cudaEventDestroy(c->ev_fork);
  if (c->ev_join) cudaEventDestroy(c->ev_join);
  msvgb_detail::tune_free(c);
  if (c->h_pin) cudaFreeHost(c->h_pin);
  if (c->h_one) cudaFreeHost(c->h_one);
  delete c;
  return MSVGB_eslOK;
}

extern "C" int msvgb_ctx_set_stream(msvgb_ctx *c, void *stream) {
  if (!c) return fail(MSVGB_eslEINVAL, "ctx is NULL");
  c->stream = stream ? (cudaStream_t) stream : c->own;
  return MSVGB_eslOK;
}

// ------------------------------------------------------------------------------
// profile: host re-layout of the striped rbv into the kernels' lane layout

static inline int rbv_at(const msvgb_om *om, int Q, int x, int k) {   // k = 1..M
  const int q = (k - 1) % Q, z = (k - 1) / Q;
  return om->rbv[((size_t) x * Q + q) * 16 + z];
}

// node held by DP word w, half h of lane l (1-based)
static inline int node_of(int C, int lane, int w, int h) { return lane * 2 * C + h * C + w + 1; }

// Builds the device tables of a profile. force_C > 0 imposes the DP width
// (the batched kernel uses a coarser set of widths); it must exceed M/64.
// Host images of a profile's device tables at DP width C: the SSV costs
// (f16x2 regions of F16Layout<C>, or int8x4) and the MSV costs (uint8x4).
int msvgb_detail::build_cost_tables(const msvgb_om *om, int f16, int C, std::vector<uint32_t> &st,
                                    std::vector<uint32_t> &mt) {
  const int M = om->M, Q = std::max(2, (M - 1) / 16 + 1), bias = om->bias_b;

  // SSV costs s = bias - rbv clamped to [-128, 127]; nodes past M and the pad
  // residue get -128, which floors every cell (u < 128) like the reference's
  // padding cost 255 / sbv 127 does.
  auto s_of = [&](int x, int k) -> int {
    if (x >= 29 || k > M) return -128;
    int s = bias - rbv_at(om, Q, x, k);
    return std::min(127, std::max(-128, s));
  };
  auto n_of = [&](int x, int k) -> int {   // MSV: 255 - rbv; padding rbv = 255 -> 0
    if (x >= 29 || k > M) return 0;
    return 255 - rbv_at(om, Q, x, k);
  };
  const int NP = (C + 1) / 2;                       // MSV table words per lane
  const size_t mwords = (size_t) NRES * NP * 32;
  const size_t swords = f16 ? (size_t) NRES * C * 32 : (size_t) NRES * (C / 2) * 32;
  st.assign(swords, 0u);
  mt.assign(mwords, 0u);
  auto f16bits = [](int v) -> uint32_t {
    const __half h = __float2half((float) v);
    uint16_t b; memcpy(&b, &h, 2); return b;
  };
  const int Q4 = C / 4, R = C % 4;
  const size_t a_words = (size_t) NRES * Q4 * 32 * 4, b_words = (R >= 2) ? (size_t) NRES * 32 * 2 : 0;
  for (int x = 0; x < NRES; ++x)
    for (int l = 0; l < 32; ++l) {
      for (int p = 0; p < NP; ++p) {
        const int w0 = 2 * p, w1 = 2 * p + 1;
        const int k0 = node_of(C, l, w0, 0), k2 = node_of(C, l, w0, 1);
        const int k1 = w1 < C ? node_of(C, l, w1, 0) : M + 1, k3 = w1 < C ? node_of(C, l, w1, 1) : M + 1;
        mt[((size_t) x * NP + p) * 32 + l] = (uint32_t) n_of(x, k0) | ((uint32_t) n_of(x, k1) << 8) |
                                            ((uint32_t) n_of(x, k2) << 16) | ((uint32_t) n_of(x, k3) << 24);
        if (!f16)
          st[((size_t) x * (C / 2) + p) * 32 + l] =
              (uint32_t) (uint8_t) s_of(x, k0) | ((uint32_t) (uint8_t) s_of(x, k1) << 8) |
              ((uint32_t) (uint8_t) s_of(x, k2) << 16) | ((uint32_t) (uint8_t) s_of(x, k3) << 24);
      }
      if (f16)
        for (int w = 0; w < C; ++w) {
          const uint32_t v = f16bits(s_of(x, node_of(C, l, w, 0))) | (f16bits(s_of(x, node_of(C, l, w, 1))) << 16);
          size_t i;                                  // F16Layout<C> in msv_device.cuh
          if (w < 4 * Q4)      i = (((size_t) x * Q4 + w / 4) * 32 + l) * 4 + (w % 4);
          else if (R >= 2 && w < 4 * Q4 + 2) i = a_words + ((size_t) x * 32 + l) * 2 + (w - 4 * Q4);
          else                 i = a_words + b_words + (size_t) x * 32 + l;
          st[i] = v;
        }
    }

  return MSVGB_eslOK;
}

// DP width and table type of a profile's 32-lane tables: f16 when asked for
// and possible, and whenever the int8 layout cannot hold M; force_C > 0
// imposes the width.
static int width_for(const msvgb_om *om, int want_f16, int force_C, int *ret_C, bool *ret_f16) {
  if (!om) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (om->M < 1) return fail(MSVGB_eslEINVAL, "profile M must be >= 1");
  if (om->Kp != 29) return fail(MSVGB_eslEINVAL, "only the amino alphabet (Kp = 29) is supported");
  if (!om->rbv) return fail(MSVGB_eslEINVAL, "rbv is NULL");
  const int c16 = force_C > 0 ? force_C : choose_C(om->M, true);
  const bool f16 = c16 > 0 && c16 <= kMaxF16C && (want_f16 || (force_C <= 0 && choose_C(om->M, false) < 0));
  const int C = force_C > 0 ? force_C : choose_C(om->M, f16);
  if (C < 0) return fail(MSVGB_eslEINVAL, "profile M exceeds the supported maximum (8191 nodes)");
  if (C < need_C(om->M) || (!f16 && (C & 1))) return fail(MSVGB_eslEINVAL, "DP width too small for M");
  *ret_C = C;
  *ret_f16 = f16;
  return MSVGB_eslOK;
}

// DP words per lane and 8-bit words per lane of the G-lane tables (G = 16 or
// 8, or 32 for the split passes of models of 1024-2047 nodes).
static int group_width(int M, int G, int *ret_C, int *ret_CI) {
  if (G != 16 && G != 8 && G != 32) return fail(MSVGB_eslEINVAL, "lanes per sequence must be 32, 16 or 8");
  const int C = M / (2 * G) + 1;                          // 2*C*G > M: the last node is padding
  if (C > 32) return fail(MSVGB_eslEINVAL, "model too long for this many lanes per sequence");
  if (C < 2) return fail(MSVGB_eslEINVAL, "model too short for this many lanes per sequence");
  int CI = msvgb_detail::hyb_default_words(C, G);
  if (CI > 0 && !msvgb_detail::hyb_compiled(C, G, CI)) CI = 0;
  *ret_C = C;
  *ret_CI = CI;
  return MSVGB_eslOK;
}

int msvgb_detail::profile_build_width(msvgb_ctx *ctx, const msvgb_om *om, int want_f16, int force_C,
                                      msvgb_profile **ret) {
  if (!om || !ret) return fail(MSVGB_eslEINVAL, "NULL argument");
  int C = 0;
  bool f16 = true;
  const int ws = width_for(om, want_f16, force_C, &C, &f16);
  if (ws != MSVGB_eslOK) return ws;
  std::vector<uint32_t> st, mt;
  build_cost_tables(om, f16 ? 1 : 0, C, st, mt);
  const size_t swords = st.size(), mwords = mt.size();
  const int M = om->M;
  msvgb_profile *p = new msvgb_profile();
  p->ctx = ctx; p->device = ctx->device; p->M = M; p->C = C; p->f16 = f16 ? 1 : 0;
  p->tbm = om->tbm_b; p->tec = om->tec_b; p->base = om->base_b; p->bias = om->bias_b;
  p->scale = om->scale_b; p->mmu = om->mmu; p->mlambda = om->mlambda;
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_stab, swords * 4);
  if (e == cudaSuccess) e = cudaMalloc(&p->d_mtab, mwords * 4);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_stab, st.data(), swords * 4, cudaMemcpyHostToDevice);
  if (e == cudaSuccess) e = cudaMemcpy(p->d_mtab, mt.data(), mwords * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    msvgb_profile_destroy(p);
    return fail(e == cudaErrorMemoryAllocation ? MSVGB_eslEMEM : MSVGB_eslESYS,
                std::string("profile upload: ") + cudaGetErrorString(e));
  }
  *ret = p;
  return MSVGB_eslOK;
}

static int profile_build(msvgb_ctx *ctx, const msvgb_om *om, int want_f16, msvgb_profile **ret) {
  return msvgb_detail::profile_build_width(ctx, om, want_f16, 0, ret);
}

static int default_f16() { return 1; }

// Lanes per sequence and SSV table type from the context's tuning table (or
// the fixed rule) for the whole length mix.
// The choice msvgb_profile_create makes for a model of M nodes: G lanes per
// sequence in the SSV pass; *split: lane-group tables are built (G < 32, or
// the split 32-lane passes of models of 1024-2047 nodes); *want_f16: the
// table type of the 32-lane tables.
static void create_choice(msvgb_ctx *ctx, int M, int *G, bool *split, int *want_f16) {
  int variant = default_f16();
  *G = M >= 1 ? msvgb_detail::lanes_for(ctx, M, -1, &variant) : 32;
  const bool wide = *G == 32 && M >= kWideSplitMinM && M / 64 + 1 <= 32;
  *split = *G < 32 || wide;
  *want_f16 = *split ? 1 : variant;
}

extern "C" int msvgb_profile_create(msvgb_ctx *ctx, const msvgb_om *om, msvgb_profile **ret) {
  if (!ctx) return fail(MSVGB_eslEINVAL, "ctx is NULL");
  if (ret) *ret = nullptr;
  if (!om) return fail(MSVGB_eslEINVAL, "om is NULL");
  int G = 32, want_f16 = 1;
  bool split = false;
  create_choice(ctx, om->M, &G, &split, &want_f16);
  int st = profile_build(ctx, om, want_f16, ret);
  if (st == MSVGB_eslOK && split && (*ret)->f16) {
    st = msvgb_profile_set_lanes(*ret, om, G);
    if (st != MSVGB_eslOK) { msvgb_profile_destroy(*ret); *ret = nullptr; }
  }
  if (st == MSVGB_eslOK) (*ret)->lanes_auto = true;
  return st;
}

extern "C" int msvgb_profile_create_ex(msvgb_ctx *ctx, const msvgb_om *om, int variant, msvgb_profile **ret) {
  if (!ctx) return fail(MSVGB_eslEINVAL, "ctx is NULL");
  if (variant != 0 && variant != 1) return fail(MSVGB_eslEINVAL, "ssv_variant must be 0 or 1");
  if (ret) *ret = nullptr;
  return profile_build(ctx, om, variant, ret);
}

extern "C" int msvgb_profile_variant(const msvgb_profile *p) { return p ? p->f16 : -1; }

extern "C" int msvgb_profile_destroy(msvgb_profile *p) {
  if (!p) return MSVGB_eslOK;
  cudaSetDevice(p->device);
  for (auto *t : p->tables) {
    cudaFree(t->d_tjb); cudaFree(t->d_xjmin);
    for (void *r : t->retired) cudaFree(r);
    delete t;
  }
  cudaFree(p->d_stab); cudaFree(p->d_mtab); cudaFree(p->d_stab_g); cudaFree(p->d_mtab_g);
  delete p;
  return MSVGB_eslOK;
}

extern "C" int msvgb_profile_M(const msvgb_profile *p) { return p ? p->M : -1; }

// G-lane f16 table (GroupLayout<C, G>, with its region copies): node
// g*2C + h*C + w + 1 of lane g in word w, half h, holding cost(x, node).
template <class Cost>
static std::vector<uint32_t> group_table_from(int C, int G, Cost cost) {
  auto f16bits = [](int v) -> uint32_t {
    const __half h = __float2half((float) v);
    uint16_t b; memcpy(&b, &h, 2); return b;
  };
  const int Q4 = C / 4, R = C % 4;
  const int pair = G < 16 ? 16 / G : 1, single = 32 / G;      // region copies (GroupCopies)
  const size_t a_words = (size_t) NRES * Q4 * G * 4, b_words = (R >= 2) ? (size_t) NRES * pair * G * 2 : 0;
  std::vector<uint32_t> st((size_t) group_words(C, G, 0));
  for (int x = 0; x < NRES; ++x)
    for (int g = 0; g < G; ++g)
      for (int w = 0; w < C; ++w) {
        const int k0 = g * 2 * C + w + 1, k1 = g * 2 * C + C + w + 1;
        const uint32_t v = f16bits(cost(x, k0)) | (f16bits(cost(x, k1)) << 16);
        if (w < 4 * Q4) {
          st[(((size_t) x * Q4 + w / 4) * G + g) * 4 + (w % 4)] = v;
        } else if (R >= 2 && w < 4 * Q4 + 2) {
          for (int cp = 0; cp < pair; ++cp) st[a_words + (((size_t) x * pair + cp) * G + g) * 2 + (w - 4 * Q4)] = v;
        } else {
          for (int cp = 0; cp < single; ++cp) st[a_words + b_words + ((size_t) x * single + cp) * G + g] = v;
        }
      }
  return st;
}

// G-lane SSV table: s = bias - rbv clamped to [-128, 127]; padding -128.
std::vector<uint32_t> msvgb_detail::build_group_table(const msvgb_om *om, int C, int G) {
  const int M = om->M, Q = std::max(2, (M - 1) / 16 + 1), bias = om->bias_b;
  return group_table_from(C, G, [&](int x, int k) -> int {
    if (x >= 29 || k > M) return -128;
    return std::min(127, std::max(-128, bias - rbv_at(om, Q, x, k)));
  });
}

// G-lane MSV table (the full recurrence, msv_row_group): c = bias - rbv
// unclamped; padding nodes and the pad residue bias - 255 (rbv 255).
std::vector<uint32_t> msvgb_detail::build_group_msv_table(const msvgb_om *om, int C, int G) {
  const int M = om->M, Q = std::max(2, (M - 1) / 16 + 1), bias = om->bias_b;
  return group_table_from(C, G, [&](int x, int k) -> int {
    if (x >= 29 || k > M) return bias - 255;
    return bias - rbv_at(om, Q, x, k);
  });
}

extern "C" int msvgb_profile_set_lanes(msvgb_profile *p, const msvgb_om *om, int G) {
  if (!p || !om) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (om->M != p->M) return fail(MSVGB_eslEINVAL, "om does not match the profile");
  p->lanes_auto = false;                                  // set by the caller: applies at any size
  // 32 lanes: the fused kernel, and for models of 1024 to 2047 nodes also
  // the split passes (32-lane groups, mixed-width SSV table), which large
  // searches use
  const bool wide = G == 32 && p->M >= kWideSplitMinM && p->M / 64 + 1 <= 32;
  if (G == 32 && !wide) {
    cudaFree(p->d_stab_g); cudaFree(p->d_mtab_g);
    p->d_stab_g = p->d_mtab_g = nullptr;
    p->G = 32; p->CI = 0;
    return MSVGB_eslOK;
  }
  int C = 0, CI = 0;
  const int gs = group_width(p->M, G, &C, &CI);
  if (gs != MSVGB_eslOK) return gs;
  std::vector<uint32_t> st = CI ? build_hyb_table(om, C, G, CI) : build_group_table(om, C, G);
  CUDA_TRY(cudaSetDevice(p->device));
  uint32_t *d = nullptr;
  CUDA_TRY(cudaMalloc(&d, st.size() * 4));
  cudaError_t e = cudaMemcpy(d, st.data(), st.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(d); return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
  const std::vector<uint32_t> mg = build_group_msv_table(om, C, G);
  uint32_t *dm = nullptr;
  e = cudaMalloc(&dm, mg.size() * 4);
  if (e == cudaSuccess) e = cudaMemcpy(dm, mg.data(), mg.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(d); cudaFree(dm); return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
  cudaFree(p->d_stab_g);
  cudaFree(p->d_mtab_g);
  p->d_stab_g = d; p->d_mtab_g = dm; p->Cg = C; p->G = G; p->CI = CI;
  return MSVGB_eslOK;
}

extern "C" int msvgb_profile_lanes(const msvgb_profile *p) { return p ? p->G : -1; }

int msvgb_detail::build_profile_tables(msvgb_ctx *ctx, const msvgb_om *om, ProfileTables &t) {
  if (!ctx || !om) return fail(MSVGB_eslEINVAL, "NULL argument");
  int G = 32, want_f16 = 1;
  bool split = false, f16 = true;
  create_choice(ctx, om->M, &G, &split, &want_f16);
  t = ProfileTables();
  int st = width_for(om, want_f16, 0, &t.C, &f16);
  if (st != MSVGB_eslOK) return st;
  t.f16 = f16 ? 1 : 0;
  build_cost_tables(om, t.f16, t.C, t.st, t.mt);
  if (split && f16) {
    st = group_width(om->M, G, &t.Cg, &t.CI);
    if (st != MSVGB_eslOK) return st;
    t.G = G;
    t.stg = t.CI ? build_hyb_table(om, t.Cg, G, t.CI) : build_group_table(om, t.Cg, G);
    t.mtg = build_group_msv_table(om, t.Cg, G);
  }
  return MSVGB_eslOK;
}

// Mixed-width lane-group table: the first C - CI words of every lane as f16
// bits of s units of 2^-24 (sign-magnitude: s < 0 -> 0x8000 | -s), the last
// CI words (a multiple of 4) as bytes t = s + 128 (layout HybLayout<C, CI, G>,
// msv_group.cuh).
std::vector<uint32_t> msvgb_detail::build_hyb_table(const msvgb_om *om, int C, int G, int CI) {
  const int M = om->M, Q = std::max(2, (M - 1) / 16 + 1), bias = om->bias_b;
  auto s_of = [&](int x, int k) -> int {
    if (x >= 29 || k > M) return -128;
    return std::min(127, std::max(-128, bias - rbv_at(om, Q, x, k)));
  };
  auto sm16 = [](int v) -> uint32_t { return v < 0 ? 0x8000u | (uint32_t) (-v) : (uint32_t) v; };
  const int CF = C - CI, Q4 = CF / 4, R = CF % 4, NO = CI / 8, HALF = (CI % 8) / 4;
  const int pair = G < 16 ? 16 / G : 1, single = 32 / G;      // region copies (GroupCopies)
  const size_t a_words = (size_t) NRES * Q4 * G * 4, b_words = (R >= 2) ? (size_t) NRES * pair * G * 2 : 0;
  const size_t c_words = (R & 1) ? (size_t) NRES * single * G : 0, d_words = (size_t) NRES * NO * G * 4;
  std::vector<uint32_t> st((size_t) group_words(C, G, CI));
  for (int x = 0; x < NRES; ++x)
    for (int g = 0; g < G; ++g) {
      auto k_of = [&](int w, int h) { return g * 2 * C + h * C + w + 1; };
      for (int w = 0; w < CF; ++w) {
        const uint32_t v = sm16(s_of(x, k_of(w, 0))) | (sm16(s_of(x, k_of(w, 1))) << 16);
        if (w < 4 * Q4) {
          st[(((size_t) x * Q4 + w / 4) * G + g) * 4 + (w % 4)] = v;
        } else if (R >= 2 && w < 4 * Q4 + 2) {
          for (int cp = 0; cp < pair; ++cp) st[a_words + (((size_t) x * pair + cp) * G + g) * 2 + (w - 4 * Q4)] = v;
        } else {
          for (int cp = 0; cp < single; ++cp) st[a_words + b_words + ((size_t) x * single + cp) * G + g] = v;
        }
      }
      auto t = [&](int ww, int h) { return (uint32_t) (s_of(x, k_of(ww, h)) + 128); };
      auto tword = [&](int w) { return t(w, 0) | (t(w + 1, 0) << 8) | (t(w, 1) << 16) | (t(w + 1, 1) << 24); };
      for (int o = 0; o < NO; ++o)
        for (int k = 0; k < 4; ++k)
          st[a_words + b_words + c_words + (((size_t) x * NO + o) * G + g) * 4 + k] = tword(CF + 8 * o + 2 * k);
      for (int k = 0; k < 2 * HALF; ++k)
        for (int cp = 0; cp < pair; ++cp)
          st[a_words + b_words + c_words + d_words + (((size_t) x * pair + cp) * G + g) * 2 + k] =
              tword(CF + 8 * NO + 2 * k);
    }
  return st;
}

extern "C" int msvgb_profile_set_ssv_int8_words(msvgb_profile *p, const msvgb_om *om, int words) {
  if (!p || !om) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (om->M != p->M) return fail(MSVGB_eslEINVAL, "om does not match the profile");
  if (p->G == 32 || !p->d_stab_g)
    return fail(MSVGB_eslEINVAL, "8-bit SSV words are set for 16 or 8 lanes per sequence (32 lanes: fixed)");
  if (words == p->CI) return MSVGB_eslOK;
  if (words != 0 && !hyb_compiled(p->Cg, p->G, words))
    return fail(MSVGB_eslEINVAL, "no mixed-width SSV kernel for this model length, lane count and word count");
  const std::vector<uint32_t> st = words ? build_hyb_table(om, p->Cg, p->G, words)
                                         : build_group_table(om, p->Cg, p->G);
  CUDA_TRY(cudaSetDevice(p->device));
  uint32_t *d = nullptr;
  CUDA_TRY(cudaMalloc(&d, st.size() * 4));
  cudaError_t e = cudaMemcpy(d, st.data(), st.size() * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) { cudaFree(d); return fail(MSVGB_eslESYS, cudaGetErrorString(e)); }
  cudaFree(p->d_stab_g);
  p->d_stab_g = d; p->CI = words;
  return MSVGB_eslOK;
}

extern "C" int msvgb_profile_ssv_int8_words(const msvgb_profile *p) { return p ? p->CI : -1; }

// ------------------------------------------------------------------------------
// per-length tables: tjb_b(L) and the smallest xJ that passes F1 at length L

int msvgb_detail::xjmin_for(const msvgb_profile *p, int L, double F1, int hint) {
  const int tjb = msvgb_tjb_b(p->scale, L);
  auto pass = [&](int xj) {
    return msvgb_f1_pass(score_from_xj(xj, tjb, p->base, p->scale), L, p->mmu, p->mlambda, F1, nullptr) != 0;
  };
  if (hint >= 0 && hint <= 255) {
    // Walk from a nearby length's answer (the boundary moves by a unit or two
    // between neighbouring lengths): down while xJ - 1 still passes, or up
    // until xJ passes. Every step evaluates the predicate on both sides of
    // the boundary it returns, as the checks below do.
    int b = hint;
    if (b == 255 || pass(b)) {
      while (b > 0 && pass(b - 1)) --b;
    } else {
      ++b;
      while (b < 255 && !pass(b)) ++b;
    }
    return b;
  }
  // P is non-increasing in xJ; binary search, then confirm the boundary.
  int lo = 0, hi = 255;                  // answer in [lo, hi]; 255 = no xJ < 255 passes
  while (lo < hi) {
    const int mid = (lo + hi) / 2;
    if (pass(mid)) hi = mid; else lo = mid + 1;
  }
  if (lo < 255 && !pass(lo)) return -1;
  if (lo > 0 && pass(lo - 1)) return -1;
  return lo;
}

int msvgb_detail::ensure_tables(msvgb_profile *p, const msvgb_db *db, double F1, LenTables **out) {
  std::lock_guard<std::mutex> lk(p->tables_mu);
  LenTables *t = nullptr;
  for (auto *x : p->tables) if (x->F1 == F1) t = x;
  if (!t) {
    if (p->tables.size() >= 8) return fail(MSVGB_eslEINVAL, "too many distinct F1 thresholds for one profile");
    t = new LenTables();
    t->F1 = F1;
    p->tables.push_back(t);
  }
  const int need = db->Lmax + 1;
  bool dirty = false;
  if (need > t->cap) {                                  // grow: host images and device buffers
    const int cap = std::max({need, 2 * t->cap, 1024});
    t->tjb.resize(cap);
    for (int L = t->cap; L < cap; ++L) t->tjb[L] = msvgb_tjb_b(p->scale, L);
    t->xjm.resize(cap, -1);
    uint8_t *nt = nullptr, *nx = nullptr;
    cudaError_t e = cudaMalloc(&nt, cap);
    if (e == cudaSuccess) e = cudaMalloc(&nx, cap);
    if (e != cudaSuccess) {
      cudaFree(nt); cudaFree(nx);
      return fail(MSVGB_eslEMEM, std::string("length tables: ") + cudaGetErrorString(e));
    }
    if (t->d_tjb) { t->retired.push_back(t->d_tjb); t->retired.push_back(t->d_xjmin); }
    t->d_tjb = nt; t->d_xjmin = nx;
    t->cap = cap;
    dirty = true;
  }
  int hint = -1;                                        // the last length's answer (lengths ascend)
  for (int L : db->distinct_len) {
    if (L == 0) continue;
    if (t->xjm[L] >= 0) { hint = t->xjm[L]; continue; }
    const int v = xjmin_for(p, L, F1, hint);
    if (v < 0) return fail(MSVGB_eslESYS, "F1 pass set is not monotone in xJ");
    t->xjm[L] = (int16_t) v;
    hint = v;
    dirty = true;
  }
  if (dirty) {
    std::vector<uint8_t> x(t->cap);
    for (int L = 0; L < t->cap; ++L) x[L] = t->xjm[L] < 0 ? 255 : (uint8_t) t->xjm[L];
    // Complete before this returns, i.e. before any later search is launched,
    // without waiting behind searches still running on the context's stream:
    // entries those may read are rewritten with the bytes they already hold
    // (or live in retired buffers), so they read consistent values.
    cudaError_t e = cudaMemcpyAsync(t->d_tjb, t->tjb.data(), t->cap, cudaMemcpyHostToDevice, p->ctx->upload);
    if (e == cudaSuccess) e = cudaMemcpyAsync(t->d_xjmin, x.data(), t->cap, cudaMemcpyHostToDevice, p->ctx->upload);
    if (e == cudaSuccess) e = cudaStreamSynchronize(p->ctx->upload);
    if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("length tables: ") + cudaGetErrorString(e));
  }
  *out = t;
  return MSVGB_eslOK;
}

// ------------------------------------------------------------------------------
// database: sort by length (longest first), pad each sequence to 16 bytes

// Host work is O(n + Lmax): a stable counting sort of the lengths (longest
// first) and the padded offsets. The residues go to the device in one copy
// (a DMA when the caller's buffer is pinned) and a kernel scatters, pads and
// validates them.
// Phase timings of msvgb_db_create on stderr when MSVGB_TRACE is set.
static bool trace_on() { static const bool on = getenv("MSVGB_TRACE") != nullptr; return on; }
struct PhaseTimer {
  std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
  void mark(const char *what) {
    if (!trace_on()) return;
    const auto now = std::chrono::steady_clock::now();
    fprintf(stderr, "msvgb: %-28s %8.3f ms\n", what, std::chrono::duration<double, std::milli>(now - t).count());
    t = now;
  }
};

extern "C" int msvgb_db_create(msvgb_ctx *ctx, const uint8_t *codes, const int64_t *off, int64_t n,
                               msvgb_db **ret) {
  if (!ctx) return fail(MSVGB_eslEINVAL, "NULL argument");
  return msvgb_detail::db_create_on(ctx, codes, off, n, ctx->stream, ret);
}

// Grows the context's small pinned scratch (no copy into it may be pending).
static cudaError_t grow_pinned(msvgb_ctx *ctx, size_t need) {
  if (ctx->h_pin) cudaFreeHost(ctx->h_pin);
  ctx->h_pin = nullptr; ctx->h_pin_cap = 0;
  need = std::max<size_t>(need, 1 << 16);
  cudaError_t e = cudaMallocHost(&ctx->h_pin, need);
  if (e == cudaSuccess) ctx->h_pin_cap = need;
  return e;
}

cudaMemPool_t msvgb_detail::scratch_pool(int device) {
  static std::mutex mu;
  static std::unordered_map<int, cudaMemPool_t> pools;
  std::lock_guard<std::mutex> lk(mu);
  auto it = pools.find(device);
  if (it != pools.end()) return it->second;
  cudaMemPoolProps props = {};
  props.allocType = cudaMemAllocationTypePinned;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = device;
  cudaMemPool_t pool = nullptr;
  if (cudaMemPoolCreate(&pool, &props) != cudaSuccess) return nullptr;
  uint64_t keep = (uint64_t) 4 << 30;
  cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
  pools[device] = pool;
  return pool;
}

// msvgb_db_create with its copies and packing on stream st. Without an
// AsyncPack it returns when the database is complete on the device. With one,
// it returns once everything is enqueued: invalid codes are OR-ed into
// a->d_bad (checked by the caller) and db->ready completes when the database
// is on the device; chunked (a->cuts), the chunks' residues are only copied,
// and pack_chunk_on packs each.
//
// The offsets go up first, then the raw residues in one DMA (one per chunk)
// on the context's dma stream. Meanwhile the lengths are sorted on the
// device: lengths and their maximum (the only value the host waits for
// before the end), counts per (chunk, length), a scan of the counts chunk by
// chunk and by descending length (first sorted slot and first packed byte of
// every key), placement; then the residues are scattered into the packed
// layout. The counts come back to the host at the end, for the distinct
// lengths the per-length tables need. Databases with sequences longer than 4M
// residues are sorted on the host instead.
int msvgb_detail::db_create_on(msvgb_ctx *ctx, const uint8_t *codes, const int64_t *off, int64_t n,
                               cudaStream_t st, msvgb_db **ret, const AsyncPack *a) {
  if (!ctx || !ret || (n > 0 && (!off || !codes))) return fail(MSVGB_eslEINVAL, "NULL argument");
  PhaseTimer pt;
  *ret = nullptr;
  if (n < 0) return fail(MSVGB_eslEINVAL, "n < 0");
  const int64_t total = n ? off[n] - off[0] : 0;
  if (total < 0) return fail(MSVGB_eslEINVAL, "bad sequence offsets");
  const bool chunked = a && a->cuts;
  ChunkCuts cuts;                                             // one chunk unless chunked
  cuts.cut[1] = n;
  if (chunked) {
    const std::vector<int64_t> &c = *a->cuts;
    if (c.size() < 2 || c.size() > (size_t) kMaxChunks + 1 || c.front() != 0 || c.back() != n)
      return fail(MSVGB_eslEINVAL, "bad chunk cuts");
    for (size_t k = 0; k + 1 < c.size(); ++k)
      if (c[k + 1] < c[k]) return fail(MSVGB_eslEINVAL, "bad chunk cuts");
    cuts.K = (int) c.size() - 1;
    for (size_t k = 0; k < c.size(); ++k) cuts.cut[k] = c[k];
  }
  const int K = cuts.K;
  CUDA_TRY(cudaSetDevice(ctx->device));
  msvgb_detail::GpuTrace gt;
  gt.mark("db: start", st);
  const int64_t n1 = std::max<int64_t>(n, 1);
  cudaMemPool_t pool = scratch_pool(ctx->device);
  if (!pool) return fail(MSVGB_eslESYS, "database upload: no memory pool");
  std::vector<void *> scratch;                                // freed on st at the end
  auto alloc = [&](void **ptr, size_t bytes, cudaStream_t s2) {
    cudaError_t r = cudaMallocFromPoolAsync(ptr, std::max<size_t>(bytes, 16), pool, s2);
    if (r == cudaSuccess) scratch.push_back(*ptr);
    return r;
  };
  int64_t *d_off = nullptr, *d_scal = nullptr;                // d_scal: [0] Lmax | bad << 32, [1] packed size
  int32_t *d_len_in = nullptr;
  uint8_t *d_raw = nullptr;
  std::vector<cudaEvent_t> chunk_up;
  cudaEvent_t ev_raw = nullptr;
  CUDA_TRY(cudaEventCreateWithFlags(&ev_raw, cudaEventDisableTiming));
  cudaError_t e = alloc((void **) &d_off, (size_t) (n + 1) * 8, st);
  if (e == cudaSuccess) e = alloc((void **) &d_len_in, (size_t) n1 * 4, st);
  if (e == cudaSuccess) e = alloc((void **) &d_scal, 16, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(d_off, off, (size_t) (n + 1) * 8, cudaMemcpyHostToDevice, st);
  gt.mark("db: offsets up", st);
  if (e == cudaSuccess) e = cudaEventRecord(ev_raw, st);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->dma, ev_raw, 0);
  if (!chunked) {
    if (e == cudaSuccess) e = alloc((void **) &d_raw, (size_t) total + 64, ctx->dma);   // slack: pack_kernel
    if (e == cudaSuccess && total) e = cudaMemcpyAsync(d_raw, codes + off[0], total, cudaMemcpyHostToDevice, ctx->dma);
    if (e == cudaSuccess) e = cudaEventRecord(ev_raw, ctx->dma);
  } else {
    // kept past this call (pack_chunk_on reads it): not scratch
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync((void **) &d_raw, (size_t) total + 64, pool, ctx->dma);
    for (int k = 0; k < K && e == cudaSuccess; ++k) {
      const int64_t r0 = off[cuts.cut[k]] - off[0], r1 = off[cuts.cut[k + 1]] - off[0];
      if (r1 > r0) e = cudaMemcpyAsync(d_raw + r0, codes + off[0] + r0, r1 - r0, cudaMemcpyHostToDevice, ctx->dma);
      cudaEvent_t ev = nullptr;
      if (e == cudaSuccess) e = cudaEventCreateWithFlags(&ev, cudaEventDisableTiming);
      if (e == cudaSuccess) { chunk_up.push_back(ev); e = cudaEventRecord(ev, ctx->dma); }
    }
  }
  auto drop_chunk_inputs = [&]() {
    for (cudaEvent_t ev : chunk_up) cudaEventDestroy(ev);
    chunk_up.clear();
    if (chunked && d_raw) { cudaStreamSynchronize(ctx->dma); cudaFreeAsync(d_raw, ctx->dma); d_raw = nullptr; }
  };
  pt.mark("copies issued");
  if (e == cudaSuccess && ctx->h_pin_cap < 64) e = grow_pinned(ctx, 64);
  unsigned *misc = (unsigned *) ctx->h_pin;
  if (e == cudaSuccess) { misc[0] = misc[1] = 0; e = cudaMemsetAsync(d_scal, 0, 16, st); }
  if (e == cudaSuccess) e = launch_lengths(d_off, n, d_len_in, (unsigned *) d_scal, (int *) d_scal + 1,
                                           ctx->num_sms, st);
  if (e == cudaSuccess) e = cudaMemcpyAsync(misc, d_scal, 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  pt.mark("lengths");
  gt.mark("db: lengths (host waited)", st);
  const bool bad_len = e == cudaSuccess && misc[1] != 0;
  const int Lmax = e == cudaSuccess ? (int) misc[0] : 0;
  auto finish = [&]() {                                       // scratch frees, ordered after all use
    cudaStreamWaitEvent(st, ev_raw, 0);
    for (void *q : scratch) cudaFreeAsync(q, st);
    scratch.clear();
    cudaEventDestroy(ev_raw);
  };
  if (e != cudaSuccess || bad_len) {
    finish();
    drop_chunk_inputs();
    cudaStreamSynchronize(st);
    if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("database upload: ") + cudaGetErrorString(e));
    return fail(MSVGB_eslEINVAL, "bad sequence offsets");
  }

  msvgb_db *db = new msvgb_db();
  db->ctx = ctx; db->device = ctx->device; db->n = n; db->residues = total; db->Lmax = Lmax;
  db->serial = g_db_serial.fetch_add(1);
  const size_t nb = (size_t) Lmax + 1;
  // the (chunk, length) keys of the device sort must fit an int and a modest table
  const bool gpu_sort = Lmax <= (1 << 22) && (size_t) K * nb <= (size_t) (1 << 24);
  // packed size: exact after a host sort, an upper bound before the device scan
  int64_t pos = 0;
  const int64_t bound = gpu_sort ? total + 15 * n : 0;
  // The database's own arrays come from the pool too: cudaMalloc would wait for
  // kernels still running (a search of an earlier chunk). msvgb_db_destroy's
  // cudaFree synchronizes before it frees them.
  auto keep = [&](void **ptr, size_t bytes) {
    return cudaMallocFromPoolAsync(ptr, std::max<size_t>(bytes, 16), pool, st);
  };
  int64_t *d_src = nullptr;
  e = chunked ? keep((void **) &d_src, (size_t) n1 * 8) : alloc((void **) &d_src, (size_t) n1 * 8, st);
  if (e == cudaSuccess) e = keep((void **) &db->d_start, (size_t) n1 * 8);
  if (e == cudaSuccess) e = keep((void **) &db->d_orig, (size_t) n1 * 8);
  if (e == cudaSuccess) e = keep((void **) &db->d_len, (size_t) n1 * 4);
  unsigned long long *d_hist = nullptr;
  std::map<std::pair<int, int32_t>, int64_t> host_hist;       // host sort: counts per (chunk, length)
  auto chunk_of = [&](int64_t i) { int k = 0; while (k + 1 < K && i >= cuts.cut[k + 1]) ++k; return k; };
  if (e == cudaSuccess && gpu_sort) {
    int64_t *d_bins = nullptr;                                // per key: first slot, then first byte; scan scratch
    e = keep((void **) &db->d_codes, bound + 64);
    if (e == cudaSuccess) e = alloc((void **) &d_hist, K * nb * 8, st);
    if (e == cudaSuccess) e = alloc((void **) &d_bins, (2 * K * nb + bins_scratch_words(Lmax, K)) * 8, st);
    uint32_t *d_blk = nullptr;                                // per part and short key: counts, then first ranks
    const size_t blk_words = (size_t) sort_parts(ctx->num_sms) * K * sort_small_bound(Lmax, K);
    if (e == cudaSuccess) e = alloc((void **) &d_blk, blk_words * 4, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(d_hist, 0, K * nb * 8, st);
    if (e == cudaSuccess) e = launch_histogram(d_len_in, n, d_hist, d_blk, cuts, Lmax, ctx->num_sms, st);
    if (e == cudaSuccess) e = launch_bins(d_hist, Lmax, K, d_bins, d_bins + K * nb, d_bins + 2 * K * nb, d_scal + 1,
                                          db->d_codes, st);
    unsigned long long *cursor = nullptr;
    if (e == cudaSuccess) e = alloc((void **) &cursor, K * nb * 8, st);
    if (e == cudaSuccess) e = cudaMemcpyAsync(cursor, d_bins, K * nb * 8, cudaMemcpyDeviceToDevice, st);
    if (e == cudaSuccess) e = launch_place(d_off, d_len_in, n, cursor, d_blk, d_bins, d_bins + K * nb, db->d_start,
                                           db->d_orig, db->d_len, d_src, cuts, Lmax, ctx->num_sms, st);
    pt.mark("sort enqueued");
    gt.mark("db: placed", st);
  } else if (e == cudaSuccess) {
    // host fallback for very long sequences: stable sort by chunk, then by
    // descending length
    std::vector<int64_t> idx(n);
    for (int64_t i = 0; i < n; ++i) idx[i] = i;
    std::stable_sort(idx.begin(), idx.end(), [&](int64_t x, int64_t y) {
      const int cx = chunk_of(x), cy = chunk_of(y);
      if (cx != cy) return cx < cy;
      return off[x + 1] - off[x] > off[y + 1] - off[y];
    });
    std::vector<int64_t> h_start(n), h_orig(n), h_src(n);
    std::vector<int32_t> h_len(n);
    for (int64_t s = 0; s < n; ++s) {
      const int64_t i = idx[s], L = off[i + 1] - off[i];
      h_orig[s] = i; h_len[s] = (int32_t) L; h_src[s] = off[i] - off[0]; h_start[s] = pos;
      pos += (L + 15) / 16 * 16;
      host_hist[{chunk_of(i), (int32_t) L}]++;
    }
    e = keep((void **) &db->d_codes, pos + 64);
    if (e == cudaSuccess) e = cudaMemsetAsync(db->d_codes + pos, PAD_CODE, 64, st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(db->d_start, h_start.data(), n * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(db->d_orig, h_orig.data(), n * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(d_src, h_src.data(), n * 8, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess && n) e = cudaMemcpyAsync(db->d_len, h_len.data(), n * 4, cudaMemcpyHostToDevice, st);
    if (e == cudaSuccess) e = cudaStreamSynchronize(st);      // the vectors above feed the copies
    pt.mark("host sort");
  }
  // scatter the residues once they are up; then the counts and flags come back
  const size_t hist_bytes = gpu_sort ? K * nb * 8 : 0;
  if (e == cudaSuccess && ctx->h_pin_cap < 16 + hist_bytes) e = grow_pinned(ctx, 16 + hist_bytes);
  int *d_bad = a ? a->d_bad : ctx->d_bad;
  int64_t *h_scal = (int64_t *) ctx->h_pin;                   // [0] bad flag, [1] packed size, then counts
  if (!chunked) {
    if (e == cudaSuccess) e = cudaStreamWaitEvent(st, ev_raw, 0);
    if (trace_on() && e == cudaSuccess) { e = cudaStreamSynchronize(st); pt.mark("residues up"); }
    if (e == cudaSuccess && !a) e = cudaMemsetAsync(d_bad, 0, sizeof(int), st);
    if (e == cudaSuccess) e = launch_pack(d_raw, d_src, db->d_start, db->d_len, n, db->d_codes, d_bad,
                                          ctx->num_sms, st);
  }
  if (e == cudaSuccess) { h_scal[0] = 0; h_scal[1] = pos; }
  if (e == cudaSuccess && !a) e = cudaMemcpyAsync(h_scal, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && gpu_sort) e = cudaMemcpyAsync(h_scal + 1, d_scal + 1, 8, cudaMemcpyDeviceToHost, st);
  if (e == cudaSuccess && gpu_sort) e = cudaMemcpyAsync(h_scal + 2, d_hist, hist_bytes, cudaMemcpyDeviceToHost, st);
  finish();
  gt.mark("db: counts back", st);
  if (e == cudaSuccess) e = cudaStreamSynchronize(st);
  pt.mark("pack");
  // distinct lengths (ascending) with their counts, over all chunks and per chunk (descending)
  db->chunk_len.assign(K, {});
  db->chunk_cnt.assign(K, {});
  if (e == cudaSuccess) {
    auto add = [&](int k, int32_t L, int64_t c) {
      db->chunk_len[k].push_back(L);
      db->chunk_cnt[k].push_back(c);
    };
    auto add_total = [&](int32_t L, int64_t c) {
      db->distinct_len.push_back(L);
      db->len_count.push_back(c);
      if (L >= kLongTarget) db->n_long += c;
    };
    if (gpu_sort) {
      pos = h_scal[1];
      const unsigned long long *hist = (const unsigned long long *) (h_scal + 2);
      // hist in sorted key order: chunk k's lengths descending from k * nb
      for (int k = 0; k < K; ++k)
        for (int r = 0; r < (int) nb; ++r)
          if (hist[(size_t) k * nb + r]) add(k, Lmax - r, (int64_t) hist[(size_t) k * nb + r]);
      for (int L = 0; L <= Lmax; ++L) {
        int64_t c = 0;
        for (int k = 0; k < K; ++k) c += (int64_t) hist[(size_t) k * nb + (Lmax - L)];
        if (c) add_total(L, c);
      }
    } else {
      std::map<int32_t, int64_t> all;
      for (auto it = host_hist.rbegin(); it != host_hist.rend(); ++it) {   // within a chunk: descending length
        add(it->first.first, it->first.second, it->second);
        all[it->first.second] += it->second;
      }
      for (const auto &v : all) add_total(v.first, v.second);
    }
  }
  gt.mark("db: counts read", nullptr);
  gt.print();
  db->packed_bytes = pos + 64;
  if (chunked) {
    db->chunk_slot.assign(cuts.cut, cuts.cut + K + 1);        // every chunk keeps its size
    db->chunk_up = chunk_up;
    chunk_up.clear();
    db->d_raw = d_raw; d_raw = nullptr;
    db->d_src = d_src;
    db->d_bad_chunks = d_bad;
  }
  if (e == cudaSuccess && a && !chunked) e = cudaEventCreateWithFlags(&db->ready, cudaEventDisableTiming);
  if (e == cudaSuccess && a && !chunked) e = cudaEventRecord(db->ready, st);
  if (e == cudaSuccess && n && !chunked) count_launch();
  if (e != cudaSuccess) {
    cudaStreamSynchronize(st);
    cudaStreamSynchronize(ctx->dma);
    drop_chunk_inputs();
    msvgb_db_destroy(db);
    return fail(e == cudaErrorMemoryAllocation ? MSVGB_eslEMEM : MSVGB_eslESYS,
                std::string("database upload: ") + cudaGetErrorString(e));
  }
  if (!a && h_scal[0]) {
    msvgb_db_destroy(db);
    return fail(MSVGB_eslEINVAL, "residue code >= 29 (Kp)");
  }
  *ret = db;
  return MSVGB_eslOK;
}

int msvgb_detail::pack_chunk_on(msvgb_ctx *ctx, msvgb_db *db, int k, cudaStream_t st) {
  if (!db->d_raw || k < 0 || k + 1 >= (int) db->chunk_slot.size()) return fail(MSVGB_eslEINVAL, "no such chunk");
  const int64_t s0 = db->chunk_slot[k], s1 = db->chunk_slot[k + 1];
  CUDA_TRY(cudaStreamWaitEvent(st, db->chunk_up[k], 0));
  if (s1 > s0) {
    CUDA_TRY(launch_pack(db->d_raw, db->d_src + s0, db->d_start + s0, db->d_len + s0, s1 - s0, db->d_codes,
                         db->d_bad_chunks, ctx->num_sms, st));
    count_launch();
  }
  return MSVGB_eslOK;
}

void msvgb_detail::release_chunks_on(msvgb_db *db, cudaStream_t st) {
  if (db->d_raw) cudaFreeAsync(db->d_raw, st);
  if (db->d_src) cudaFreeAsync(db->d_src, st);
  db->d_raw = nullptr;
  db->d_src = nullptr;
}

void msvgb_detail::db_release_on(msvgb_db *db, cudaStream_t st) {
  if (!db) return;
  cudaSetDevice(db->device);
  for (void *q : {(void *) db->d_codes, (void *) db->d_start, (void *) db->d_orig, (void *) db->d_len,
                  (void *) db->d_raw, (void *) db->d_src, (void *) db->d_inv})
    if (q) cudaFreeAsync(q, st);
  for (cudaEvent_t ev : db->chunk_up) cudaEventDestroy(ev);
  if (db->ready) cudaEventDestroy(db->ready);
  delete db;
}

extern "C" int msvgb_db_destroy(msvgb_db *db) {
  if (!db) return MSVGB_eslOK;
  cudaSetDevice(db->device);
  cudaFree(db->d_codes); cudaFree(db->d_start); cudaFree(db->d_orig); cudaFree(db->d_len);
  cudaFree(db->d_raw); cudaFree(db->d_src);
  for (cudaEvent_t ev : db->chunk_up) cudaEventDestroy(ev);
  if (db->ready) cudaEventDestroy(db->ready);
  cudaFree(db->d_inv);
  delete db;
  return MSVGB_eslOK;
}
extern "C" int64_t msvgb_db_nseq(const msvgb_db *db) { return db ? db->n : -1; }
extern "C" int64_t msvgb_db_residues(const msvgb_db *db) { return db ? db->residues : -1; }

// ------------------------------------------------------------------------------
// search

extern "C" int msvgb_search_device(msvgb_ctx *c, const msvgb_profile *pc, const msvgb_db *db, double F1,
                                   void *d_xj, void *d_flags) {
  if (!c || !pc || !db || (!d_xj && db->n) || (!d_flags && db->n)) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (pc->ctx != c || db->ctx != c) return fail(MSVGB_eslEINVAL, "objects belong to another context");
  if (db->n == 0) return MSVGB_eslOK;
  msvgb_profile *p = const_cast<msvgb_profile *>(pc);
  CUDA_TRY(cudaSetDevice(c->device));
  LenTables *t = nullptr;
  int st = ensure_tables(p, db, F1, &t);
  if (st != MSVGB_eslOK) return st;
  if (db->ready) CUDA_TRY(cudaStreamWaitEvent(c->stream, db->ready, 0));   // still being packed
  if (c->list_cap < (size_t) db->n) {
    CUDA_TRY(cudaStreamSynchronize(c->stream));            // the old list may still be read
    cudaFree(c->d_list); c->d_list = nullptr; c->list_cap = 0;
    CUDA_TRY(cudaMalloc(&c->d_list, sizeof(int64_t) * db->n));
    c->list_cap = db->n;
  }
  SearchScratch sc;
  sc.stream = c->stream; sc.side = c->side; sc.ev_fork = c->ev_fork; sc.ev_join = c->ev_join;
  sc.ticket = c->d_ticket; sc.aux = c->d_aux; sc.list = c->d_list;
  return enqueue_search(sc, p, db, t, (uint8_t *) d_xj, (uint8_t *) d_flags, c->num_sms);
}

int msvgb_detail::enqueue_search(const SearchScratch &sc, const msvgb_profile *p, const msvgb_db *db,
                                 const LenTables *t, uint8_t *d_xj, uint8_t *d_flags, int num_sms) {
  DbDev dbv{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  ProfDev P32;
  P32.M = p->M; P32.C = p->C; P32.tbm = p->tbm; P32.tec = p->tec; P32.base = p->base; P32.bias = p->bias;
  P32.stab = p->d_stab; P32.mtab = p->d_mtab; P32.tjb = t->d_tjb; P32.xjmin = t->d_xjmin; P32.ssv_f16 = p->f16;
  // Lane groups lengthen each sequence's latency (2-4x): below ~40 G cells the
  // launch tail they add outweighs their throughput, unless lanes were set
  // explicitly.
  const bool small = p->lanes_auto && (double) p->M * (double) db->residues < 4e10;
  if (!p->d_stab_g || small) {
    LaunchArgs a;
    a.P = P32; a.db = dbv; a.out_xj = d_xj; a.out_flags = d_flags; a.ticket = sc.ticket;
    a.stream = sc.stream; a.grid = 0; a.skip_empty = 1;
    CUDA_TRY(cudaMemsetAsync(sc.ticket, 0, sizeof(unsigned long long), sc.stream));
    CUDA_TRY(dispatch(p->C, p->f16 != 0, a, num_sms));
    count_launch();
    return MSVGB_eslOK;
  }
  // Long targets (they sort first) on the 32-lane kernel, in the side stream
  // when there is one; the rest: the G-lane SSV pass, then the full MSV on the
  // sequences it left undecided. The side stream forks from and joins back
  // into the search's. Targets too long for a lane group to finish within the
  // pass go to 32 lanes: with the longest first, a group's latency only
  // matters beyond about a third of the rows each group scores on average
  // (SMs x 32 warps x 32/G groups), and never below kLongTarget residues.
  const double groups = (double) num_sms * 32.0 * (32.0 / p->G);
  const int t_long = (int) std::min<double>(1e9, std::max<double>(kLongTarget, (double) db->residues / groups / 3.0));
  const int64_t n_long = std::min(db->count_at_least(t_long), db->n);
  ProfDev P;
  P.M = p->M; P.C = p->Cg; P.tbm = p->tbm; P.tec = p->tec; P.base = p->base; P.bias = p->bias;
  P.stab = p->d_stab_g; P.mtab = p->d_mtab; P.tjb = t->d_tjb; P.xjmin = t->d_xjmin; P.ssv_f16 = 1;
  GroupArgs g;
  g.P = P; g.db = dbv; g.out_xj = d_xj; g.out_flags = d_flags;
  g.ticket = sc.ticket; g.undecided = sc.list; g.n_undecided = sc.aux + 1; g.stream = sc.stream;
  g.s_begin = n_long;
  CUDA_TRY(cudaMemsetAsync(sc.ticket, 0, sizeof(unsigned long long), sc.stream));
  CUDA_TRY(cudaMemsetAsync(sc.aux, 0, 3 * sizeof(unsigned long long), sc.stream));
  if (n_long > 0) {
    LaunchArgs l;
    l.P = P32; l.db = dbv; l.out_xj = d_xj; l.out_flags = d_flags; l.ticket = sc.aux + 2;
    l.stream = sc.side ? sc.side : sc.stream; l.grid = 0; l.skip_empty = 1; l.range_end = n_long;
    if (sc.side) {
      CUDA_TRY(cudaEventRecord(sc.ev_fork, sc.stream));
      CUDA_TRY(cudaStreamWaitEvent(sc.side, sc.ev_fork, 0));
    }
    CUDA_TRY(dispatch(p->C, p->f16 != 0, l, num_sms));
    count_launch();
    if (sc.side) CUDA_TRY(cudaEventRecord(sc.ev_join, sc.side));
  }
  if (n_long < db->n) {
    CUDA_TRY(dispatch_group(p->Cg, p->G, p->CI, g, num_sms));
    count_launch();
  }
  if (p->d_mtab_g) {                                       // the full MSV on the same lane groups
    ProfDev Pl = P;
    Pl.mtab = p->d_mtab_g;
    CUDA_TRY(dispatch_list_group(p->Cg, p->G, Pl, dbv, d_xj, d_flags, sc.aux, sc.list, sc.aux + 1, num_sms,
                                 sc.stream));
  } else {
    LaunchArgs a;
    a.P = P32; a.db = dbv; a.out_xj = d_xj; a.out_flags = d_flags; a.ticket = sc.aux;
    a.stream = sc.stream; a.grid = 0; a.skip_empty = 1; a.list = sc.list; a.list_count = sc.aux + 1;
    CUDA_TRY(dispatch(p->C, p->f16 != 0, a, num_sms));
  }
  count_launch();
  if (n_long > 0 && sc.side) CUDA_TRY(cudaStreamWaitEvent(sc.stream, sc.ev_join, 0));
  return MSVGB_eslOK;
}

extern "C" int msvgb_search(msvgb_ctx *c, const msvgb_profile *p, const msvgb_db *db, double F1,
                            uint8_t *out_xj, uint8_t *out_flags) {
  if (!c || !p || !db || (db->n && (!out_xj || !out_flags))) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (db->n == 0) return MSVGB_eslOK;
  CUDA_TRY(cudaSetDevice(c->device));
  uint8_t *d = nullptr;
  CUDA_TRY(cudaMallocAsync((void **) &d, 2 * (size_t) db->n, c->stream));
  int st = msvgb_search_device(c, p, db, F1, d, d + db->n);
  if (st == MSVGB_eslOK) {
    cudaError_t e = cudaMemcpyAsync(out_xj, d, db->n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_flags, d + db->n, db->n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
    if (e != cudaSuccess) st = fail(MSVGB_eslESYS, std::string("search: ") + cudaGetErrorString(e));
  }
  cudaFreeAsync(d, c->stream);
  if (st == MSVGB_eslOK) CUDA_TRY(cudaStreamSynchronize(c->stream));
  return st;
}

// The search of a chunked database (db_create_on with cuts), chunk by chunk
// as each chunk's residues arrive, on two streams taken in turn (S[0] the
// context's stream, S[1] its upload stream): the chunk is packed, then its
// long targets run on the 32-lane kernel and the rest in the lane-group SSV
// pass (or everything in the 32-lane kernel for small searches and profiles
// without lane groups). A chunk's packing and start fill the SMs the previous
// chunk's pass leaves in its tail. All chunks append to one undecided list,
// scored by one full-MSV pass at the end, on S[0].
// ctr: 6 zeroed counters (per-stream tickets for the long and main passes,
// the list count, the list ticket); list: room for db->n entries.
static int search_chunked(msvgb_ctx *c, const msvgb_profile *p, msvgb_db *db, const LenTables *t, uint8_t *d_xj,
                          uint8_t *d_flags, unsigned long long *ctr, int64_t *list, msvgb_detail::GpuTrace &gt) {
  using namespace msvgb_detail;
  const int sms = c->num_sms;
  cudaStream_t S[2] = {c->stream, c->upload};
  const DbDev full{db->d_codes, db->d_start, db->d_len, db->d_orig, db->n};
  ProfDev P32;
  P32.M = p->M; P32.C = p->C; P32.tbm = p->tbm; P32.tec = p->tec; P32.base = p->base; P32.bias = p->bias;
  P32.stab = p->d_stab; P32.mtab = p->d_mtab; P32.tjb = t->d_tjb; P32.xjmin = t->d_xjmin; P32.ssv_f16 = p->f16;
  // as in enqueue_search: lane groups only where the whole search is large
  const bool small = p->lanes_auto && (double) p->M * (double) db->residues < 4e10;
  const bool groups = p->d_stab_g && !small;
  ProfDev P = P32;
  int t_long = INT32_MAX;
  if (groups) {
    P.C = p->Cg; P.stab = p->d_stab_g; P.ssv_f16 = 1;
    const double ngroups = (double) sms * 32.0 * (32.0 / p->G);
    t_long = (int) std::min<double>(1e9, std::max<double>(kLongTarget, (double) db->residues / ngroups / 3.0));
  }
  const int K = (int) db->chunk_slot.size() - 1;
  for (int k = 0; k < K; ++k) {
    cudaStream_t s = S[k & 1];
    unsigned long long *tk_long = ctr + (k & 1), *tk = ctr + 2 + (k & 1);
    int st = pack_chunk_on(c, db, k, s);
    if (st != MSVGB_eslOK) return st;
    gt.mark("chunk " + std::to_string(k) + " packed", s);
    const int64_t s0 = db->chunk_slot[k], s1 = db->chunk_slot[k + 1];
    if (s1 == s0) continue;
    const DbDev part{db->d_codes, db->d_start + s0, db->d_len + s0, db->d_orig + s0, s1 - s0};
    const int64_t n_long = groups ? std::min(db->chunk_count_at_least(k, t_long), s1 - s0) : s1 - s0;
    if (n_long > 0) {                                       // 32 lanes: long targets, or the whole chunk
      LaunchArgs l;
      l.P = P32; l.db = part; l.out_xj = d_xj; l.out_flags = d_flags; l.ticket = tk_long;
      l.stream = s; l.grid = 0; l.skip_empty = 1; l.range_end = n_long;
      CUDA_TRY(cudaMemsetAsync(tk_long, 0, sizeof(unsigned long long), s));
      CUDA_TRY(dispatch(p->C, p->f16 != 0, l, sms));
      count_launch();
    }
    if (groups && s0 + n_long < s1) {
      GroupArgs g;
      g.P = P; g.db = full; g.db.n = s1; g.out_xj = d_xj; g.out_flags = d_flags;
      g.ticket = tk; g.undecided = list; g.n_undecided = ctr + 4; g.stream = s; g.s_begin = s0 + n_long;
      CUDA_TRY(cudaMemsetAsync(tk, 0, sizeof(unsigned long long), s));
      CUDA_TRY(dispatch_group(p->Cg, p->G, p->CI, g, sms));
      count_launch();
    }
    gt.mark("chunk " + std::to_string(k) + " passed", s);
  }
  CUDA_TRY(cudaEventRecord(c->ev_join, S[1]));
  CUDA_TRY(cudaStreamWaitEvent(S[0], c->ev_join, 0));
  release_chunks_on(db, S[0]);
  if (groups) {                                             // the full MSV of the undecided sequences
    if (p->d_mtab_g) {
      ProfDev Pl = P;
      Pl.mtab = p->d_mtab_g;
      CUDA_TRY(dispatch_list_group(p->Cg, p->G, Pl, full, d_xj, d_flags, ctr + 5, list, ctr + 4, sms, S[0]));
    } else {
      LaunchArgs a;
      a.P = P32; a.db = full; a.out_xj = d_xj; a.out_flags = d_flags; a.ticket = ctr + 5;
      a.stream = S[0]; a.grid = 0; a.skip_empty = 1; a.list = list; a.list_count = ctr + 4;
      CUDA_TRY(dispatch(p->C, p->f16 != 0, a, sms));
    }
    count_launch();
    gt.mark("list passed", S[0]);
  }
  return MSVGB_eslOK;
}

// End to end from host buffers. The input is cut into chunks of consecutive
// sequences and sorted once, chunk by chunk (search_chunked). Its offsets go
// up first and then every chunk's residues, back to back on the copy engine;
// the first chunk is small, so that its search starts as soon as the sort
// ends, and the copy (at ~4x the rate the search consumes residues) stays
// ahead of the search from then on. Results land in one device buffer and
// come back in one copy at the end.
int msvgb_detail::host_search(msvgb_ctx *c, const msvgb_profile *pc, const uint8_t *codes, const int64_t *off,
                              int64_t n, double F1, int64_t chunk_residues, uint8_t *out_xj, uint8_t *out_flags,
                              msvgb_db **keep_db) {
  if (keep_db) *keep_db = nullptr;
  if (!c || !pc || n < 0 || (n && (!codes || !off || !out_xj || !out_flags)))
    return fail(MSVGB_eslEINVAL, "NULL argument");
  if (pc->ctx != c) return fail(MSVGB_eslEINVAL, "objects belong to another context");
  if (n == 0 && !keep_db) return MSVGB_eslOK;
  if (n == 0) return db_create_on(c, codes, off, 0, c->stream, keep_db);
  msvgb_profile *p = const_cast<msvgb_profile *>(pc);
  msvgb_detail::GpuTrace gt;
  CUDA_TRY(cudaSetDevice(c->device));
  // chunk boundaries: chunks growing from a quarter of chunk_residues to it
  // (by default a third of the residues: a first chunk of a twelfth, whose
  // copy ends about when the sort does, then a sixth, then thirds, the
  // remainder last); one chunk below kOneChunkResidues, where the whole copy
  // is shorter than the sort. At most kMaxChunks.
  std::vector<int64_t> cut(1, 0);
  const int64_t total = off[n] - off[0];
  constexpr int64_t kOneChunkResidues = 64 << 20;
  const bool one = chunk_residues <= 0 && total < kOneChunkResidues;
  if (chunk_residues <= 0) chunk_residues = one ? std::max<int64_t>(1, total) : total / 3 + 1;
  int64_t want = one ? std::max<int64_t>(1, total) : std::max<int64_t>(1, chunk_residues / 4);
  for (int64_t b0 = 0; b0 < n;) {
    // the first sequence boundary at least want residues past b0's start, or n
    int64_t b1 = std::lower_bound(off + b0 + 1, off + n, off[b0] + want) - off;
    if ((int) cut.size() == kMaxChunks) b1 = n;               // the last chunk takes the rest
    cut.push_back(b1);
    b0 = b1;
    want = std::min(chunk_residues, 2 * want);
  }
  gt.mark("chunks cut", nullptr);
  // device scratch: results [xj n | flags n], the invalid-code flag, 6 counters; the undecided list
  const size_t o_bad = (2 * (size_t) n + 15) / 16 * 16, o_ctr = o_bad + 16;
  uint8_t *d = nullptr;
  int64_t *d_list = nullptr;
  CUDA_TRY(cudaMallocAsync((void **) &d, o_ctr + 6 * sizeof(unsigned long long), c->stream));
  int *d_bad = (int *) (d + o_bad);
  unsigned long long *ctr = (unsigned long long *) (d + o_ctr);
  cudaError_t e = cudaMallocAsync((void **) &d_list, sizeof(int64_t) * (size_t) n, c->stream);
  if (e == cudaSuccess) e = cudaMemsetAsync(d + o_bad, 0, 16 + 6 * sizeof(unsigned long long), c->stream);
  if (e == cudaSuccess) e = cudaEventRecord(c->ev_fork, c->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(c->upload, c->ev_fork, 0);   // scratch ready before any pack
  if (e != cudaSuccess) {
    cudaFreeAsync(d_list, c->stream);
    cudaFreeAsync(d, c->stream);
    cudaStreamSynchronize(c->stream);
    return fail(MSVGB_eslESYS, std::string("search: ") + cudaGetErrorString(e));
  }
  gt.mark("start", c->stream);
  PhaseTimer pt;
  msvgb_db *db = nullptr;
  AsyncPack a{d_bad};
  a.cuts = &cut;
  int st = db_create_on(c, codes, off, n, c->upload, &db, &a);
  gt.mark("sorted", c->upload);
  pt.mark("search_host: sorted");
  LenTables *t = nullptr;
  if (st == MSVGB_eslOK) st = ensure_tables(p, db, F1, &t);
  if (st == MSVGB_eslOK) st = search_chunked(c, p, db, t, d, d + n, ctr, d_list, gt);
  pt.mark("search_host: enqueued");
  int bad = 0;
  if (st == MSVGB_eslOK) {
    e = cudaMemcpyAsync(out_xj, d, n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(out_flags, d + n, n, cudaMemcpyDeviceToHost, c->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, c->stream);
    if (e != cudaSuccess) st = fail(MSVGB_eslESYS, std::string("search: ") + cudaGetErrorString(e));
  }
  cudaStreamSynchronize(c->upload);
  cudaStreamSynchronize(c->dma);
  cudaFreeAsync(d_list, c->stream);
  cudaFreeAsync(d, c->stream);
  e = cudaStreamSynchronize(c->stream);
  pt.mark("search_host: done");
  gt.mark("results back", c->stream);
  if (st == MSVGB_eslOK && e != cudaSuccess) st = fail(MSVGB_eslESYS, std::string("search: ") + cudaGetErrorString(e));
  if (st == MSVGB_eslOK && bad) st = fail(MSVGB_eslEINVAL, "residue code >= 29 (Kp)");
  if (keep_db && st == MSVGB_eslOK) {                       // packed and complete: the stream was synchronized
    db->d_bad_chunks = nullptr;                               // pointed into this call's scratch
    *keep_db = db;
  }
  else msvgb_db_destroy(db);
  gt.mark("database kept or freed", nullptr);
  gt.print();
  return st;
}

extern "C" int msvgb_search_host(msvgb_ctx *c, const msvgb_profile *p, const uint8_t *codes, const int64_t *off,
                                 int64_t n, double F1, int64_t chunk_residues, uint8_t *out_xj,
                                 uint8_t *out_flags) {
  return msvgb_detail::host_search(c, p, codes, off, n, F1, chunk_residues, out_xj, out_flags, nullptr);
}

// ------------------------------------------------------------------------------
// drop-in single call

static uint64_t fnv1a(const void *data, size_t n, uint64_t h) {
  const uint8_t *b = (const uint8_t *) data;
  for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ull; }
  return h;
}

// The bytes a drop-in profile's device tables are built from: the scalar MSV
// fields (tjb_b excluded: the caller rewrites it per target length) and the
// rbv vectors.
static void om_image(const msvgb_om *om, std::vector<uint8_t> &img) {
  const int Q = std::max(2, (om->M - 1) / 16 + 1);
  const size_t nrbv = (size_t) om->Kp * Q * 16;
  img.resize(16 + nrbv);
  uint8_t *b = img.data();
  memcpy(b, &om->M, 4);
  memcpy(b + 4, &om->Kp, 4);
  b[8] = om->tbm_b; b[9] = om->tec_b; b[10] = om->base_b; b[11] = om->bias_b;
  memcpy(b + 12, &om->scale_b, 4);
  memcpy(b + 16, om->rbv, nrbv);
}

// Whether om's bytes equal a cached image (no copy: header then rbv).
static bool om_equals(const msvgb_om *om, const std::vector<uint8_t> &img) {
  const int Q = std::max(2, (om->M - 1) / 16 + 1);
  const size_t nrbv = (size_t) om->Kp * Q * 16;
  if (img.size() != 16 + nrbv) return false;
  uint8_t h[16];
  memcpy(h, &om->M, 4);
  memcpy(h + 4, &om->Kp, 4);
  h[8] = om->tbm_b; h[9] = om->tec_b; h[10] = om->base_b; h[11] = om->bias_b;
  memcpy(h + 12, &om->scale_b, 4);
  return memcmp(h, img.data(), 16) == 0 && memcmp(om->rbv, img.data() + 16, nrbv) == 0;
}

// The cached profile for om, or a new one. A cache entry is found by the
// caller's rbv pointer and M first (the usual case: the same P7_OPROFILE, or
// clones sharing its vectors), else by content hash; either way its bytes are
// compared with om's before it is used, so neither a reused pointer nor a hash
// collision can score om with another profile's tables.
static int dropin_profile(msvgb_ctx *c, const msvgb_om *om, msvgb_profile **ret) {
  DropinEntry *hit = nullptr;
  for (auto &e : c->dropin)
    if (e.rbv_ptr == om->rbv && e.M == om->M && om_equals(om, e.image)) { hit = &e; break; }
  if (!hit) {
    const int Q = std::max(2, (om->M - 1) / 16 + 1);
    uint64_t h = 1469598103934665603ull;
    const uint8_t hdr[5] = {om->tbm_b, om->tec_b, om->base_b, om->bias_b, (uint8_t) om->Kp};
    h = fnv1a(&om->M, sizeof(int), h);
    h = fnv1a(hdr, sizeof(hdr), h);
    h = fnv1a(&om->scale_b, sizeof(float), h);
    h = fnv1a(om->rbv, (size_t) om->Kp * Q * 16, h) & c->hash_mask;
    for (auto &e : c->dropin)
      if (e.hash == h && om_equals(om, e.image)) { hit = &e; break; }
    if (hit) {
      hit->rbv_ptr = om->rbv;                                  // the fast path finds it next time
    } else {
      msvgb_profile *p = nullptr;
      const int st = profile_build(c, om, default_f16(), &p);
      if (st != MSVGB_eslOK) return st;
      if (c->dropin.size() >= 64) {                            // evict the least recently used
        auto lru = std::min_element(c->dropin.begin(), c->dropin.end(),
                                    [](const DropinEntry &a, const DropinEntry &b) { return a.last_use < b.last_use; });
        msvgb_profile_destroy(lru->p);
        c->dropin.erase(lru);
      }
      DropinEntry e;
      e.rbv_ptr = om->rbv; e.M = om->M; e.hash = h; e.p = p;
      om_image(om, e.image);
      c->dropin.push_back(std::move(e));
      hit = &c->dropin.back();
    }
  }
  hit->last_use = ++c->dropin_clock;
  *ret = hit->p;
  return MSVGB_eslOK;
}

extern "C" int msvgb_MSVFilter(msvgb_ctx *c, const uint8_t *dsq, int L, const msvgb_om *om, msvgb_omx *ox,
                               float *ret_sc) {
  if (!c || !dsq || !om || !ox || !ret_sc) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (om->M < 1 || !om->rbv) return fail(MSVGB_eslEINVAL, "bad profile");
  const int Q = std::max(2, (om->M - 1) / 16 + 1);
  if (Q > ox->allocQ16) return fail(MSVGB_eslEINVAL, "DP matrix allocated too small");   // msvfilter.c:103
  ox->M = om->M;
  if (L < 0) return fail(MSVGB_eslEINVAL, "L < 0");
  for (int i = 1; i <= L; ++i)
    if (dsq[i] >= 29) return fail(MSVGB_eslEINVAL, "residue code >= 29 (Kp)");
  std::lock_guard<std::mutex> lock(c->mu);
  CUDA_TRY(cudaSetDevice(c->device));
  msvgb_profile *p = nullptr;
  int st = dropin_profile(c, om, &p);
  if (st != MSVGB_eslOK) return st;
  // One block, staged in pinned memory and uploaded in one copy:
  // [0, 64) ticket (zero) and the one-sequence database arrays (start = 0,
  // orig = 0, len); [64, 64 + T) the tjb table (the caller's om->tjb_b at
  // index L, the reference reads om->tjb_b as set) then the xjmin table (255:
  // the pass flag is unused here); then the residues padded to 16 bytes with
  // the pad code.
  const size_t T = ((2 * ((size_t) L + 1)) + 15) / 16 * 16;
  const size_t padded = ((size_t) L + 15) / 16 * 16 + 64;
  const size_t bytes = 64 + T + padded;
  if (c->h_one_cap < bytes || c->d_one_cap < bytes) {
    CUDA_TRY(cudaStreamSynchronize(c->stream));               // nothing still reads the old blocks
    const size_t cap = std::max<size_t>(bytes, 16384);
    if (c->h_one) cudaFreeHost(c->h_one);
    cudaFree(c->d_one);
    c->h_one = nullptr; c->d_one = nullptr; c->h_one_cap = c->d_one_cap = 0;
    CUDA_TRY(cudaMallocHost((void **) &c->h_one, cap));
    c->h_one_cap = cap;
    CUDA_TRY(cudaMalloc((void **) &c->d_one, cap));
    c->d_one_cap = cap;
  }
  uint8_t *h = c->h_one;
  memset(h, 0, 64);
  const int32_t len32 = L;
  memcpy(h + 32, &len32, 4);                                  // [8,16) start = 0, [16,24) orig = 0, [32,36) len
  memset(h + 64, 0, T);
  h[64 + L] = om->tjb_b;
  h[64 + (L + 1) + L] = 255;
  uint8_t *hs = h + 64 + T;
  if (L) memcpy(hs, dsq + 1, (size_t) L);
  memset(hs + L, PAD_CODE, padded - (size_t) L);
  uint8_t *d = c->d_one;
  CUDA_TRY(cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, c->stream));
  const DbDev dbv{d + 64 + T, (const int64_t *) (d + 8), (const int32_t *) (d + 32), (const int64_t *) (d + 16), 1};
  ProfDev P;
  P.M = p->M; P.C = p->C; P.tbm = p->tbm; P.tec = p->tec; P.base = p->base; P.bias = p->bias;
  P.stab = p->d_stab; P.mtab = p->d_mtab; P.tjb = d + 64; P.xjmin = d + 64 + L + 1; P.ssv_f16 = p->f16;
  LaunchArgs a;
  a.P = P; a.db = dbv; a.out_xj = c->d_out; a.out_flags = c->d_out + 1;
  a.ticket = (unsigned long long *) d;
  a.stream = c->stream; a.grid = 1; a.skip_empty = 0;
  CUDA_TRY(dispatch(p->C, p->f16 != 0, a, c->num_sms));
  g_launches.fetch_add(1);
  uint8_t *res = h;                                           // the results come back into the staged block
  CUDA_TRY(cudaMemcpyAsync(res, c->d_out, 2, cudaMemcpyDeviceToHost, c->stream));
  CUDA_TRY(cudaStreamSynchronize(c->stream));
  if (res[1] & MSVGB_FLAG_ERANGE) { *ret_sc = INFINITY; return MSVGB_eslERANGE; }
  *ret_sc = score_from_xj(res[0], om->tjb_b, om->base_b, om->scale_b);
  return MSVGB_eslOK;
}
