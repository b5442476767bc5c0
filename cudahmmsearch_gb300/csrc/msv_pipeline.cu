// msv_pipeline.cu -- the hmmsearch driver's threading around the GPU MSV stage.
//
// The reference driver (src/hmmsearch.c:1317-1406; the fork's
// code/src/cudaHmmsearch.cu:670-810) has a reader thread filling blocks of
// sequences and worker threads running p7_Pipeline on each; the fork gave the
// MSV filter of a block to the GPU and ran p7_PipelineShort (p7_pipeline.c:887)
// on the rest. Here: the calling thread is the GPU submitter -- it uploads
// and scores one block after another -- while N CPU workers take each scored
// block, compute the MSV score of every sequence that passes the F1 gate
// (with the reference's exact expression) and hand it to the caller's
// continuation (the place p7_PipelineShort plugs in: bias filter, Viterbi,
// Forward, domain definition). Upload and search of block k+1 overlap the CPU
// work on block k.
#include <atomic>
#include <cmath>
#include <condition_variable>
#include <deque>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"

using msvgb_detail::fail;

namespace {

struct Block {
  int64_t b0 = 0, b1 = 0;
  std::vector<uint8_t> xj, fl;
};

}  // namespace

extern "C" int msvgb_pipeline_run(msvgb_ctx *ctx, const msvgb_om *om, const uint8_t *codes, const int64_t *off,
                                  int64_t n, int64_t block_size, double F1, int n_workers,
                                  msvgb_survivor_fn fn, void *user, int64_t *ret_n_past_msv) {
  if (!ctx || !om || (n > 0 && (!codes || !off)) || block_size < 1 || n < 0)
    return fail(MSVGB_eslEINVAL, "msvgb_pipeline_run: bad arguments");
  if (n_workers < 1) n_workers = 1;
  msvgb_profile *prof = nullptr;
  int st = msvgb_profile_create(ctx, om, &prof);
  if (st != MSVGB_eslOK) return st;

  std::mutex mu;
  std::condition_variable cv_push, cv_pop;
  std::deque<Block *> q;
  const size_t qcap = 2;                       // blocks scored ahead of the workers
  bool producing = true;
  std::atomic<int64_t> n_past{0};
  std::atomic<int> abort_flag{0};

  auto worker = [&]() {
    for (;;) {
      Block *b = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv_pop.wait(lk, [&] { return !q.empty() || !producing; });
        if (q.empty()) return;
        b = q.front();
        q.pop_front();
      }
      cv_push.notify_one();
      for (int64_t i = b->b0; i < b->b1 && !abort_flag.load(); ++i) {
        const uint8_t xj = b->xj[i - b->b0], fl = b->fl[i - b->b0];
        if (!(fl & MSVGB_FLAG_PASS)) continue;              // P > F1: rejected by the MSV stage
        const int L = (int) (off[i + 1] - off[i]);
        const float usc = msvgb_score(xj, fl, L, om->base_b, om->scale_b);
        n_past.fetch_add(1);
        if (fn && fn(user, i, usc, xj, fl) != 0) abort_flag.store(1);
      }
      delete b;
    }
  };
  std::vector<std::thread> workers;
  for (int t = 0; t < n_workers; ++t) workers.emplace_back(worker);

  // GPU submitter: upload + score one block after another
  for (int64_t b0 = 0; b0 < n && st == MSVGB_eslOK && !abort_flag.load(); b0 += block_size) {
    const int64_t b1 = std::min(n, b0 + block_size);
    Block *blk = new Block();
    blk->b0 = b0; blk->b1 = b1;
    blk->xj.resize(b1 - b0); blk->fl.resize(b1 - b0);
    msvgb_db *db = nullptr;
    st = msvgb_db_create(ctx, codes, off + b0, b1 - b0, &db);
    if (st == MSVGB_eslOK) st = msvgb_search(ctx, prof, db, F1, blk->xj.data(), blk->fl.data());
    msvgb_db_destroy(db);
    if (st != MSVGB_eslOK) { delete blk; break; }
    {
      std::unique_lock<std::mutex> lk(mu);
      cv_push.wait(lk, [&] { return q.size() < qcap; });
      q.push_back(blk);
    }
    cv_pop.notify_one();
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    producing = false;
  }
  cv_pop.notify_all();
  for (auto &t : workers) t.join();
  for (Block *b : q) delete b;
  msvgb_profile_destroy(prof);
  if (ret_n_past_msv) *ret_n_past_msv = n_past.load();
  if (st == MSVGB_eslOK && abort_flag.load()) return fail(MSVGB_eslFAIL, "the continuation asked to stop");
  return st;
}

// ---- the filter stages after MSV on the GPU -----------------------------------------

namespace {

struct HitBlock {
  std::vector<msvgb_filter_hit> hits;
};

// The bias and Viterbi stages of one block (sequences b0 .. b0 + nb of the
// caller's arrays, resident as db). keep: local indices and MSV scores of the
// F1 survivors. Appends the sequences past the last stage to out.
int filter_block(msvgb_ctx *ctx, const msvgb_filters *f, msvgb_vprofile *vp, const msvgb_db *db, int64_t b0,
                 const int64_t *off, const std::vector<int64_t> &keep, const std::vector<float> &usc,
                 msvgb_filter_stats &stats, std::vector<msvgb_filter_hit> &out, msvgb_detail::GpuTrace &gt) {
  const std::string tag = "b" + std::to_string(b0) + " ";
  const size_t ns = keep.size();
  std::vector<float> fsc(ns), nsc(ns);
  std::vector<double> P(ns);
  for (size_t j = 0; j < ns; ++j) nsc[j] = msvgb_null_score((int) (off[b0 + keep[j] + 1] - off[b0 + keep[j]]));
  if (f->compo) {
    gt.mark(tag + "bias start", ctx->stream);
    int st = msvgb_biasfilter(ctx, f->compo, f->om->M, db, keep.data(), (int64_t) ns, fsc.data());
    if (st != MSVGB_eslOK) return st;
    gt.mark(tag + "bias done", ctx->stream);
  } else {
    fsc = nsc;                                                   // --nobias: filtersc = nullsc
  }
  std::vector<size_t> past;                                      // indices into keep
  for (size_t j = 0; j < ns; ++j)
    if (msvgb_stage_pass(usc[j], fsc[j], f->om->mmu, f->om->mlambda, f->F1, &P[j])) past.push_back(j);
  stats.n_past_bias += (int64_t) past.size();
  gt.mark(tag + "bias gate", nullptr);
  std::vector<int64_t> vids;
  std::vector<size_t> vpos;
  auto hit = [&](size_t j, float vfsc) {
    msvgb_filter_hit h;
    h.seq_index = b0 + keep[j];
    h.usc = usc[j]; h.nullsc = nsc[j]; h.filtersc = fsc[j]; h.vfsc = vfsc;
    out.push_back(h);
  };
  for (size_t j : past) {
    if (f->vom && P[j] > f->F2) { vids.push_back(keep[j]); vpos.push_back(j); }
    else hit(j, NAN);                                            // Viterbi skipped: counts as passed
  }
  if (!f->vom) return MSVGB_eslOK;
  int64_t passed = (int64_t) (past.size() - vids.size());
  if (!vids.empty()) {
    std::vector<int> xc(vids.size());
    std::vector<uint8_t> vst(vids.size());
    gt.mark(tag + "vit start", ctx->stream);
    int st = msvgb_vitfilter(ctx, vp, db, vids.data(), (int64_t) vids.size(), xc.data(), vst.data());
    if (st != MSVGB_eslOK) return st;
    gt.mark(tag + "vit done", ctx->stream);
    for (size_t t = 0; t < vids.size(); ++t) {
      const size_t j = vpos[t];
      const int L = (int) (off[b0 + keep[j] + 1] - off[b0 + keep[j]]);
      const float vfsc = msvgb_vit_score(xc[t], vst[t], L, f->vom);
      if (msvgb_stage_pass(vfsc, fsc[j], f->vmu, f->vlambda, f->F2, nullptr)) {
        hit(j, vfsc);
        ++passed;
      }
    }
  }
  stats.n_past_vit += passed;
  gt.mark(tag + "vit gate", nullptr);
  return MSVGB_eslOK;
}

}  // namespace

extern "C" int msvgb_filter_collect(void *user, const msvgb_filter_hit *hit) {
  msvgb_filter_sink *s = static_cast<msvgb_filter_sink *>(user);
  const int64_t at = __atomic_fetch_add(&s->n, (int64_t) 1, __ATOMIC_RELAXED);
  if (at < s->cap) s->hits[at] = *hit;
  return 0;
}

namespace {

// A block scored by the MSV stage, waiting for the filter stages.
struct MsvBlock {
  int64_t b0 = 0, nb = 0;
  msvgb_db *db = nullptr;
  std::vector<uint8_t> xj, fl;
};

}  // namespace

// Three kinds of threads: the caller uploads and MSV-searches block after
// block on its context; one filter thread runs the bias and Viterbi stages of
// each scored block on a second context (its own stream), so block k's
// filter kernels overlap block k+1's upload and search on the GPU; the
// workers run the continuation on the hits.
extern "C" int msvgb_pipeline_filters(msvgb_ctx *ctx, const msvgb_filters *f, const uint8_t *codes,
                                      const int64_t *off, int64_t n, int64_t block_size, int n_workers,
                                      msvgb_filter_fn fn, void *user, msvgb_filter_stats *ret_stats) {
  if (!ctx || !f || !f->om || (n > 0 && (!codes || !off)) || block_size < 1 || n < 0)
    return fail(MSVGB_eslEINVAL, "msvgb_pipeline_filters: bad arguments");
  if (f->vom && f->vom->M != f->om->M) return fail(MSVGB_eslEINVAL, "MSV and Viterbi parts of different models");
  if (n_workers < 1) n_workers = 1;
  msvgb_detail::GpuTrace gt;
  msvgb_ctx *fctx = nullptr;
  msvgb_profile *prof = nullptr;
  msvgb_vprofile *vp = nullptr;
  int st = msvgb_ctx_create(ctx->device, &fctx);
  if (st == MSVGB_eslOK) st = msvgb_profile_create(ctx, f->om, &prof);
  if (st == MSVGB_eslOK && f->vom) st = msvgb_vprofile_create(fctx, f->vom, &vp);
  if (st != MSVGB_eslOK) {
    msvgb_profile_destroy(prof);
    msvgb_ctx_destroy(fctx);
    return st;
  }

  msvgb_filter_stats stats{};
  gt.mark("set up", nullptr);
  std::mutex mu;
  std::condition_variable cv;                 // any change of the two queues or the flags below
  std::deque<MsvBlock *> scored;              // MSV stage -> filter thread
  std::deque<HitBlock *> hits;                // filter thread -> workers
  const size_t qcap = 2;
  bool msv_done = false, filters_done = false;
  std::atomic<int> abort_flag{0};
  int fst = MSVGB_eslOK;                      // the filter thread's status and message
  std::string fmsg;

  auto filter_thread = [&]() {
    for (;;) {
      MsvBlock *b = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return !scored.empty() || msv_done; });
        if (scored.empty()) break;
        b = scored.front();
        scored.pop_front();
      }
      cv.notify_all();
      HitBlock *hb = new HitBlock();
      int s2 = MSVGB_eslOK;
      if (!abort_flag.load()) {
        std::vector<int64_t> keep;
        std::vector<float> usc;
        stats.nseqs += b->nb;
        stats.nres += off[b->b0 + b->nb] - off[b->b0];
        const uint8_t *fl = b->fl.data();
        for (int64_t i = 0; i < b->nb; ++i) {
          if (!(fl[i] & MSVGB_FLAG_PASS)) continue;                 // P > F1 at the MSV stage (or empty)
          const int L = (int) (off[b->b0 + i + 1] - off[b->b0 + i]);
          if (L == 0) continue;
          keep.push_back(i);
          usc.push_back(msvgb_score(b->xj[i], fl[i], L, f->om->base_b, f->om->scale_b));
        }
        stats.n_past_msv += (int64_t) keep.size();
        gt.mark("b" + std::to_string(b->b0) + " survivors listed", nullptr);
        s2 = filter_block(fctx, f, vp, b->db, b->b0, off, keep, usc, stats, hb->hits, gt);
      }
      msvgb_detail::db_release_on(b->db, fctx->stream);   // after its filter stages, without a device-wide wait
      delete b;
      if (s2 != MSVGB_eslOK) {
        delete hb;
        std::lock_guard<std::mutex> lk(mu);
        fst = s2;
        fmsg = msvgb_last_error();                                   // thread-local: carried to the caller
        abort_flag.store(1);
        cv.notify_all();
        continue;                                                    // drain the queue
      }
      std::unique_lock<std::mutex> lk(mu);
      cv.wait(lk, [&] { return hits.size() < qcap; });
      hits.push_back(hb);
      cv.notify_all();
    }
    std::lock_guard<std::mutex> lk(mu);
    filters_done = true;
    cv.notify_all();
  };
  auto worker = [&]() {
    for (;;) {
      HitBlock *b = nullptr;
      {
        std::unique_lock<std::mutex> lk(mu);
        cv.wait(lk, [&] { return !hits.empty() || filters_done; });
        if (hits.empty()) return;
        b = hits.front();
        hits.pop_front();
      }
      cv.notify_all();
      for (const msvgb_filter_hit &h : b->hits) {
        if (abort_flag.load()) break;
        if (fn && fn(user, &h) != 0) abort_flag.store(1);
      }
      delete b;
    }
  };
  std::thread ft(filter_thread);
  std::vector<std::thread> workers;
  for (int t = 0; t < n_workers; ++t) workers.emplace_back(worker);

  // MSV stage: upload and score one block after another
  for (int64_t b0 = 0; b0 < n && st == MSVGB_eslOK && !abort_flag.load(); b0 += block_size) {
    MsvBlock *b = new MsvBlock();
    b->b0 = b0;
    b->nb = std::min(n, b0 + block_size) - b0;
    b->xj.resize(b->nb);
    b->fl.resize(b->nb);
    // the block's residues go up chunk by chunk under its own search; the
    // packed block stays resident for the bias and Viterbi stages
    gt.mark("b" + std::to_string(b0) + " msv start", ctx->stream);
    st = msvgb_detail::host_search(ctx, prof, codes, off + b0, b->nb, f->F1, 0, b->xj.data(), b->fl.data(), &b->db);
    gt.mark("b" + std::to_string(b0) + " msv done", ctx->stream);
    if (st != MSVGB_eslOK) {
      msvgb_db_destroy(b->db);
      delete b;
      break;
    }
    std::unique_lock<std::mutex> lk(mu);
    cv.wait(lk, [&] { return scored.size() < qcap || abort_flag.load(); });
    scored.push_back(b);
    cv.notify_all();
  }
  {
    std::lock_guard<std::mutex> lk(mu);
    msv_done = true;
  }
  cv.notify_all();
  ft.join();
  for (auto &t : workers) t.join();
  gt.mark("continuation done", nullptr);
  for (MsvBlock *b : scored) { msvgb_db_destroy(b->db); delete b; }
  for (HitBlock *b : hits) delete b;
  msvgb_vprofile_destroy(vp);
  msvgb_profile_destroy(prof);
  msvgb_ctx_destroy(fctx);
  gt.mark("torn down", nullptr);
  gt.print();
  if (ret_stats) *ret_stats = stats;
  if (st == MSVGB_eslOK && fst != MSVGB_eslOK) return fail(fst, fmsg);
  if (st == MSVGB_eslOK && abort_flag.load()) return fail(MSVGB_eslFAIL, "the continuation asked to stop");
  return st;
}
