/* msvgb.h -- C ABI of the GB300 MSV filter (HMMER3 hmmsearch stage 1).
 *
 * Plain C: pointers, sizes and status codes only. Status codes are Easel's
 * (easel/easel.h:95-114): eslOK 0, eslEOF 3, eslEMEM 5, eslENOTFOUND 6,
 * eslEFORMAT 7, eslEINCOMPAT 10, eslEINVAL 11, eslESYS 12, eslERANGE 16,
 * eslEWRITE 27. No function calls exit(); a CUDA failure returns eslESYS and
 * msvgb_last_error() describes it.
 *
 * Residues are Easel digital codes 0..28 for the amino alphabet
 * (easel/esl_alphabet.c:275); 255 (eslDSQ_SENTINEL) only at dsq[0], dsq[L+1]
 * in the single-call entry point.
 *
 * Results are bit-exact with the reference CPU p7_MSVFilter
 * (src/impl_sse/msvfilter.c:77-213, SSV first, src/impl_sse/ssvfilter.c:1364-1413):
 * the same uint8 xJ, the same float score (+inf on overflow) and the same
 * F1 pass flag of the p7_Pipeline MSV stage (src/p7_pipeline.c:662-677).
 */
#ifndef MSVGB_H
#define MSVGB_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define MSVGB_eslOK      0
#define MSVGB_eslFAIL    1
#define MSVGB_eslEOF     3
#define MSVGB_eslEMEM    5
#define MSVGB_eslENOTFOUND 6
#define MSVGB_eslEFORMAT 7
#define MSVGB_eslEINCOMPAT 10
#define MSVGB_eslEINVAL 11
#define MSVGB_eslESYS   12
#define MSVGB_eslERANGE 16
#define MSVGB_eslEWRITE 27

/* Per-(profile, sequence) result flags written by the search entry points. */
#define MSVGB_FLAG_ERANGE 0x01  /* score overflowed: +inf (eslERANGE)                      */
#define MSVGB_FLAG_PASS   0x02  /* passes the MSV-stage F1 P-value gate                    */
#define MSVGB_FLAG_FULL   0x04  /* SSV was undecided; the full MSV recurrence ran          */
#define MSVGB_FLAG_EMPTY  0x08  /* L == 0: skipped, as p7_Pipeline does (p7_pipeline.c:662) */

/* Read-only view of the MSV fields of a P7_OPROFILE (src/impl_sse/impl_sse.h:77-87).
 * rbv is the striped [Kp][Q][16] uint8 table with Q = max(2, ceil(M/16)):
 * byte z of vector q for residue x holds the biased cost of node k = q+1+z*Q
 * (src/impl_sse/p7_oprofile.c:619-635); pass om->rbv[0] (the vectors are contiguous). */
typedef struct {
  int            M;
  int            Kp;        /* 29 (amino) */
  const uint8_t *rbv;
  uint8_t        tbm_b, tec_b, tjb_b, base_b, bias_b;
  float          scale_b;
  float          mmu, mlambda;   /* om->evparam[p7_MMU], om->evparam[p7_MLAMBDA] */
} msvgb_om;

/* The part of P7_OMX that p7_MSVFilter reads and writes (impl_sse.h:185-199). */
typedef struct {
  int allocQ16;
  int M;
} msvgb_omx;

/* Objects created on a context (profiles, databases) may be destroyed before
 * or after it; searches need their context alive.
 * Threads: a context serves one call at a time (its stream and scratch are
 * shared by its calls), except msvgb_MSVFilter, which serialises itself;
 * give each thread its own context. Profiles, ViterbiFilter profiles and
 * databases of one device may be used from several contexts at once. */
typedef struct msvgb_ctx     msvgb_ctx;      /* one GPU, one stream, device buffers   */
typedef struct msvgb_profile msvgb_profile;  /* a profile resident in HBM             */
typedef struct msvgb_db      msvgb_db;       /* a packed sequence database in HBM     */

/* ---- context ---------------------------------------------------------------- */
int         msvgb_ctx_create(int device, msvgb_ctx **ret_ctx);
int         msvgb_ctx_destroy(msvgb_ctx *ctx);
/* Launch on an external cudaStream_t (passed as void*); NULL restores the context's own. */
int         msvgb_ctx_set_stream(msvgb_ctx *ctx, void *cuda_stream);
const char *msvgb_last_error(void);
/* Count of kernels this library has launched in the calling process. */
uint64_t    msvgb_kernel_launches(void);

/* ---- drop-in single call -----------------------------------------------------
 * Replaces p7_MSVFilter(dsq, L, om, ox, ret_sc) (src/impl_sse/impl_sse.h:327,
 * src/impl_sse/msvfilter.c:78). dsq[1..L] are codes, dsq[0], dsq[L+1] sentinels.
 * om->tjb_b must already hold the value for this L (p7_oprofile_ReconfigLength),
 * as the reference requires. Returns eslOK or eslERANGE (*ret_sc = +inf);
 * eslEINVAL if p7O_NQB(om->M) > ox->allocQ16 (msvfilter.c:103). Sets ox->M = om->M.
 * The profile is uploaded once per context and cached (up to 64 profiles,
 * least recently used out), found by the caller's rbv pointer and M or by a
 * content hash and confirmed byte for byte before use. Each call then makes
 * one host-to-device copy (from pinned staging), one launch and one 2-byte
 * copy back, and waits for them. Thread-safe (serialised per context). */
int msvgb_MSVFilter(msvgb_ctx *ctx, const uint8_t *dsq, int L, const msvgb_om *om,
                    msvgb_omx *ox, float *ret_sc);

/* ---- resident profile and database --------------------------------------------
 * Upload replaces the device side of p7_oprofile_Convert's MSV part
 * (src/impl_sse/p7_oprofile.c:601-640, mf_conversion; sf_conversion :549-590):
 * the striped rbv bytes are re-laid for the kernels. om->tjb_b is ignored here:
 * the search recomputes it per target length (p7_oprofile_ReconfigMSVLength,
 * p7_oprofile.c:920-925). The SSV table type and lanes per sequence are the
 * context's choice for M (msvgb_tune_lanes; see msvgb_autotune). */
int msvgb_profile_create(msvgb_ctx *ctx, const msvgb_om *om, msvgb_profile **ret_prof);
/* Same with an explicit SSV arithmetic variant and 32 lanes per sequence:
 * 0 = int8 cost table, packed 16-bit integer cells; 1 = f16 cost table, f16x2
 * cells (exact on these integers; used where its 2x larger table fits in
 * shared memory, otherwise variant 0 is used). msvgb_profile_variant() tells
 * which. */
int msvgb_profile_create_ex(msvgb_ctx *ctx, const msvgb_om *om, int ssv_variant, msvgb_profile **ret_prof);
int msvgb_profile_variant(const msvgb_profile *prof);
/* Lanes per sequence of the SSV pass: 32 (one warp per sequence, SSV
 * and full MSV in one kernel; for models of 1024 to 2047 nodes, searches of
 * at least ~40e9 cells -- or any search, when lanes are set here -- run the
 * SSV pass and the full MSV as two launches on 32-lane groups instead, with
 * the mixed-width table), or 16 / 8 (2 / 4 sequences per warp in
 * lockstep, for small models: each lane then holds more DP words per row);
 * with 16 or 8 the sequences SSV leaves undecided are finished by the full
 * MSV in a second launch on the same lane groups, and targets of 2400 residues or more run at 32
 * lanes in a concurrent launch (one long target must not set the length of
 * the search). om must be the profile's own MSV fields. Needs M < 64 * G and,
 * for G < 32, M >= 2 * G. Lanes chosen by msvgb_profile_create apply to
 * searches of at least ~40e9 cells (M x residues); smaller ones run at 32
 * lanes, where the shorter per-sequence latency wins; lanes set here always
 * apply. */
int msvgb_profile_set_lanes(msvgb_profile *prof, const msvgb_om *om, int lanes);
int msvgb_profile_lanes(const msvgb_profile *prof);
/* Mixed-width SSV cost table of the 16- or 8-lane pass (no reference
 * counterpart): the last `words` DP words of every lane (a multiple of 4,
 * 0 = none) keep their costs as single bytes, widened in registers; the rest
 * stay 16-bit. Fewer shared-memory bytes per cell, more instructions; results
 * are identical. eslEINVAL when the profile runs at 32 lanes (fixed: 8 words
 * where the 32-lane split passes apply) or no kernel is compiled for
 * (DP width, lanes, words). msvgb_profile_set_lanes (and so
 * msvgb_profile_create) sets the default for the model length and lane
 * count: 4 or 8 words from 10 DP words per lane up, measured 4-10% faster
 * than all-16-bit costs. */
int msvgb_profile_set_ssv_int8_words(msvgb_profile *prof, const msvgb_om *om, int words);
int msvgb_profile_ssv_int8_words(const msvgb_profile *prof);

/* ---- lane-count autotuner (no reference counterpart: the SSE filter has one
 * layout) ------------------------------------------------------------------
 * Times the SSV pass at 32 lanes per sequence (f16 and int8 cost tables), 16
 * and 8 lanes on this context's GPU for a ladder of model lengths (24..1000)
 * and four target-length bins ([0,150) [150,600) [600,2400) [2400,inf)), on
 * synthetic sequences, within about budget_s seconds (<= 0: 60 s); keeps the
 * fastest choice per (M, bin) (timed in the batched kernel) and for a
 * lognormal length mix (timed on the single-query path) in the context.
 * Afterwards msvgb_profile_create, msvgb_batch_create and the server take
 * their lane counts from it; before, a fixed rule applies (8 lanes for
 * 16 <= M < 480; for M < 1024, 16 on the length mix and on targets shorter
 * than 600 in the batched kernel; else 32). */
int msvgb_autotune(msvgb_ctx *ctx, double budget_s);
/* Text form of the context's table (device name and SM count in the header). */
int msvgb_tune_save(msvgb_ctx *ctx, const char *path);
/* eslENOTFOUND: no file; eslEFORMAT: not a table; eslEINCOMPAT: measured on
 * another GPU model. */
int msvgb_tune_load(msvgb_ctx *ctx, const char *path);
/* Lanes per sequence the context chooses for model length M and target length
 * L (L < 0: the whole length mix); *ret_variant (may be NULL) gets the SSV
 * table type for 32 lanes (1 f16, 0 int8). */
int msvgb_tune_lanes(msvgb_ctx *ctx, int M, int L, int *ret_variant);

/* ---- the stage after MSV: p7_ViterbiFilter (src/impl_sse/vitfilter.c:84-250) ------
 * The ViterbiFilter part of a P7_OPROFILE (src/impl_sse/impl_sse.h:88-96) as
 * vf_conversion stores it (src/impl_sse/p7_oprofile.c:653-760): Q8 =
 * max(2, ceil(M/8)); twv = 8*Q8 vectors of 8 int16 (per q: BM MM IM DM MD MI
 * II, then the Q8 DD vectors), rwv = Kp*Q8 vectors; element z of vector q is
 * node q+1+z*Q8; xw[E,N,J,C][MOVE,LOOP] as configured (the N/J/C move cost is
 * recomputed per target length, p7_oprofile_ReconfigRestLength). */
typedef struct {
  int            M;
  int            Kp;                 /* 29 (amino) */
  const int16_t *twv;
  const int16_t *rwv;
  int16_t        xw[4][2];
  float          scale_w, nj;
  int16_t        base_w, ddbound_w;
} msvgb_vom;
typedef struct msvgb_vprofile msvgb_vprofile;
/* Models up to 8192 nodes (above 1536 the DP row lives in shared memory). */
int msvgb_vprofile_create(msvgb_ctx *ctx, const msvgb_vom *vom, msvgb_vprofile **ret);
int msvgb_vprofile_destroy(msvgb_vprofile *vp);
/* p7_ViterbiFilter on the listed sequences of db (ids: original indices, e.g.
 * the MSV survivors): out_xc[j] the final xC, out_status[j] 0 ok, 1 overflow
 * (eslERANGE: +inf), 2 empty. One warp per sequence; bit-exact with the
 * reference's int16 saturating filter, lazy F included. */
int msvgb_vitfilter(msvgb_ctx *ctx, msvgb_vprofile *vp, const msvgb_db *db, const int64_t *ids, int64_t nids,
                    int *out_xc, uint8_t *out_status);
/* The filter score in nats from xC (vitfilter.c:240-247, exact float
 * expressions) and the per-length N/J/C move cost. */
float   msvgb_vit_score(int xc, int status, int L, const msvgb_vom *vom);
int16_t msvgb_vit_move_cost(float scale_w, float nj, int L);

/* ---- the bias filter: p7_bg_FilterScore (src/p7_bg.c:473-483) -----------------
 * The composition-bias filter HMM of p7_bg_SetFilter(bg, M, compo)
 * (src/p7_bg.c:431-453; compo: the model's mean residue composition, the
 * first 20 floats of P7_OPROFILE compo) with p7_bg_SetLength's per-sequence
 * transition, scored with esl_hmm_Forward (easel/esl_hmm.c:351-409) on the
 * listed sequences of db (ids: original indices): out_sc[j] the filter null
 * score in nats (0 for an empty sequence), bit-exact with the reference's
 * float arithmetic. One thread per sequence. */
int   msvgb_biasfilter(msvgb_ctx *ctx, const float *compo, int M, const msvgb_db *db, const int64_t *ids,
                       int64_t nids, float *out_sc);
/* The length term p7_bg_FilterScore adds to the Forward score of length L. */
float msvgb_bias_length_term(float fwd, int L);
/* p7_bg_NullOne at length L (src/p7_bg.c:359-363). */
float msvgb_null_score(int L);
/* The gate of every filter stage of p7_Pipeline (src/p7_pipeline.c:673-675,
 * 684-686, 699-701): P = esl_gumbel_surv((sc - base) / log(2), mu, lambda),
 * with the pipeline's float seq_score; 1 if P <= F. */
int   msvgb_stage_pass(float sc, float base, double mu, double lambda, double F, double *ret_P);

/* ---- on-disk formats ------------------------------------------------------------
 * Pressed MSV profiles (.h3f, the MSV file hmmpress writes: HMMER 3/f binary,
 * x86-64 little-endian). Replaces p7_oprofile_ReadMSV (src/impl_sse/io.c:233)
 * for an hmmscan-style many-profile batch. Amino profiles only. */
typedef struct msvgb_h3f msvgb_h3f;
int msvgb_h3f_open(const char *path, msvgb_h3f **ret);
/* The next record's MSV fields: om->rbv points at storage owned by the reader
 * until the next read or close; mmu, mlambda come from the record's evparam;
 * name (may be NULL) receives up to name_cap - 1 bytes of the model name.
 * Returns 3 (eslEOF) after the last record; eslEFORMAT on a corrupted or
 * older-format record; eslEINCOMPAT for a non-amino model. */
int msvgb_h3f_read(msvgb_h3f *f, msvgb_om *om, char *name, int name_cap);
int msvgb_h3f_close(msvgb_h3f *f);
/* The record last read: its model composition (20 floats, P7_OPROFILE compo)
 * and evparam VMU, VLAMBDA -- what the bias filter and the ViterbiFilter gate
 * need besides the .h3p part (any pointer may be NULL). */
int msvgb_h3f_filter_params(const msvgb_h3f *f, float *compo, float *vmu, float *vlambda);
/* The rest of a pressed profile (.h3p, p7_oprofile_Write's second file,
 * impl_sse/io.c:122-170, read back by p7_oprofile_ReadRest): the next
 * record's ViterbiFilter part into vom (vom->twv, vom->rwv point at storage
 * owned by the reader until the next read or close); the annotation and
 * Forward/Backward fields are checked for length and skipped. eslEOF after
 * the last record; eslEFORMAT on a corrupted record. */
typedef struct msvgb_h3p msvgb_h3p;
int msvgb_h3p_open(const char *path, msvgb_h3p **ret);
int msvgb_h3p_read(msvgb_h3p *f, msvgb_vom *vom, char *name, int name_cap);
int msvgb_h3p_close(msvgb_h3p *f);
/* Writes (append != 0: appends) one record in the same format, as
 * p7_oprofile_Write does (io.c:89); the SSV table is derived from rbv
 * (sf_conversion, p7_oprofile.c:549-590); evparam holds mmu and mlambda only. */
int msvgb_h3f_write(const char *path, const msvgb_om *om, const char *name, int append);

/* FASTA files read into digital amino codes, as Easel's FASTA reader
 * (easel/esl_sqio_ascii.c) digitizes them: letters of
 * "ACDEFGHIKLMNPQRSTVWY-BJZOUX*~" in either case, '_' and '.' as gaps, blanks
 * skipped; any other character is eslEFORMAT. Replaces esl_sqio_ReadBlock
 * (easel/esl_sqio.c:1040) as the feed of msvgb_db_create. */
typedef struct msvgb_seqs msvgb_seqs;
int            msvgb_fasta_read(const char *path, msvgb_seqs **ret);
int64_t        msvgb_seqs_n(const msvgb_seqs *s);
const uint8_t *msvgb_seqs_codes(const msvgb_seqs *s);     /* concatenated codes */
const int64_t *msvgb_seqs_offsets(const msvgb_seqs *s);   /* n + 1 offsets into the codes */
const char    *msvgb_seqs_name(const msvgb_seqs *s, int64_t i);
int            msvgb_seqs_free(msvgb_seqs *s);

/* The packed database (length-sorted, 16-byte-aligned residues, as
 * msvgb_db_create lays it out in HBM) saved to a file and loaded back with
 * plain copies: a database is packed once, replacing the fork's offline
 * dbsort step. Loading checks every index a kernel uses; a file that fails is
 * eslEFORMAT. */
int msvgb_db_save(const msvgb_db *db, const char *path);
int msvgb_db_load(msvgb_ctx *ctx, const char *path, msvgb_db **ret);
/* Sequence lengths in the caller's original order (out: n entries). */
int msvgb_db_lengths(const msvgb_db *db, int32_t *out);
int msvgb_profile_destroy(msvgb_profile *prof);
int msvgb_profile_M(const msvgb_profile *prof);

/* Packs n sequences (codes[off[i] .. off[i+1]), no sentinels) into HBM:
 * sorted by length (longest first), each padded to 16 bytes. Replaces the
 * fork's loadDBQuad/loadCUDA host packing (code/src/GPUFunction.cu:219-255,
 * 332-415) and its offline dbsort/hmmsort length sort. Codes must be < 29. */
int     msvgb_db_create(msvgb_ctx *ctx, const uint8_t *codes, const int64_t *off, int64_t n,
                        msvgb_db **ret_db);
int     msvgb_db_destroy(msvgb_db *db);
int64_t msvgb_db_nseq(const msvgb_db *db);
int64_t msvgb_db_residues(const msvgb_db *db);

/* ---- search ---------------------------------------------------------------------
 * Plain path: one profile per launch. For every sequence i of db (original
 * order) writes out_xj[i] (final uint8 xJ; 255 on overflow) and out_flags[i]
 * (MSVGB_FLAG_*), with the pass flag at P-value threshold F1 (default 0.02,
 * src/p7_pipeline.c:210). Host output buffers; returns after the copy. */
int msvgb_search(msvgb_ctx *ctx, const msvgb_profile *prof, const msvgb_db *db, double F1,
                 uint8_t *out_xj, uint8_t *out_flags);

/* Same, outputs left in device memory (d_xj, d_flags: n bytes each, device
 * pointers), asynchronous on the context's stream. */
int msvgb_search_device(msvgb_ctx *ctx, const msvgb_profile *prof, const msvgb_db *db, double F1,
                        void *d_xj, void *d_flags);

/* End to end from host buffers, for a database that is not kept resident:
 * sequences codes[off[i] .. off[i+1]) (as msvgb_db_create takes them) are cut
 * into chunks of consecutive sequences growing from a quarter of
 * chunk_residues to it (by default a third of the residues, or one chunk
 * below 64 M residues; at most 16 chunks); the offsets
 * go up and are sorted chunk by chunk while the chunks' residues follow, and
 * every chunk is packed and searched as soon as it is up, the full MSV of all
 * chunks' undecided sequences last. Results as msvgb_search; eslEINVAL for a
 * code >= 29 (found while packing). Pinned host buffers make every copy a
 * direct DMA. The batched pre-pass the fork's p7_PipelineShort consumed
 * (src/p7_pipeline.c:887-929), with the upload hidden behind the search. */
int msvgb_search_host(msvgb_ctx *ctx, const msvgb_profile *prof, const uint8_t *codes, const int64_t *off,
                      int64_t n, double F1, int64_t chunk_residues, uint8_t *out_xj, uint8_t *out_flags);

/* ---- profile preparation ----------------------------------------------------------
 * Sample a random profile HMM of M nodes exactly as HMMER's p7_hmm_Sample does
 * with esl_randomness_Create(seed) (src/p7_hmm.c:877-918), configure its match
 * scores against the amino background (p7_ProfileConfig, src/modelconfig.c:165-176)
 * and convert them to the MSV bytes (mf_conversion, src/impl_sse/p7_oprofile.c:601-640).
 * rbv must hold Kp * max(2, ceil(M/16)) * 16 = 29 * Q * 16 bytes; om->rbv points
 * to it. om->mlambda and *ret_lambda get p7_Lambda (src/evalues.c:186-192);
 * om->mmu is left 0 until msvgb_calibrate. Host only. */
int msvgb_sample_om(uint32_t seed, int M, uint8_t *rbv, msvgb_om *om, double *ret_lambda);
/* p7_MSVMu (src/evalues.c:240-283) with p7_Calibrate's default RNG and sizes
 * (esl_randomness_CreateFast(42), 200 sequences of length 200): scores them
 * with this library's GPU search and sets om->mmu (and om->mlambda = lambda). */
int msvgb_calibrate(msvgb_ctx *ctx, msvgb_om *om, double lambda);


/* ---- allocation-free search ------------------------------------------------------
 * No counterpart in the reference. For callers that cannot allocate device
 * memory once they are running: a process whose GPU memory is all owned by
 * another allocator, or a latency-bound loop that bans cudaMalloc after
 * start-up (it can synchronise the device and can fail under memory
 * pressure). Create the profile and database at set-up time, then call this
 * with output buffers (n bytes each, device pointers) you already own; the
 * call itself calls no cudaMalloc, cudaFree or other allocating routine.
 * Its scratch (the work ticket and the per-length tables msvgb_search would
 * allocate) is one static device array of about 129 KiB that every GPU
 * loading this library keeps until the process exits, so sequences longer
 * than MSVGB_STATIC_MAX_LEN are rejected with eslEINVAL. All calls share that
 * array: calls whose work overlaps on the GPU (different streams, or
 * different host threads) race and must be serialised by the caller. The
 * first call on a device looks up the array's device address
 * (cudaGetSymbolAddress) and keeps it for the process; do not call this
 * again after a cudaDeviceReset. Work is enqueued on cuda_stream (NULL: the context's
 * stream); the two per-length tables go up from pageable host memory, so the
 * call first waits for the stream's earlier work. It always runs the fused
 * 32-lane search kernel (the lane-group pass that msvgb_search_device may
 * choose needs a database-sized list); results equal msvgb_search_device's. */
#define MSVGB_STATIC_MAX_LEN 65535
int msvgb_search_static(const msvgb_profile *prof, const msvgb_db *db, double F1,
                        void *d_xj, void *d_flags, void *cuda_stream);

/* ---- batched search: many profiles, one persistent launch ------------------------
 * All nprof profiles against db in a single persistent kernel over a
 * (profile, sequence-chunk) work queue (profiles above 2047 nodes, up to
 * 8191, get their own launches in the same graph), captured once as a CUDA graph;
 * each msvgb_batch_run replays it asynchronously on the context's stream.
 * Outputs are device buffers of nprof * n bytes, profile-major:
 * d_xj[p * n + i], d_flags[p * n + i] as msvgb_search writes them.
 * The stock hmmsearch scores one query at a time (src/hmmsearch.c:356-560);
 * this is the multi-query form of its MSV stage. */
typedef struct msvgb_batch msvgb_batch;
int     msvgb_batch_create(msvgb_ctx *ctx, const msvgb_om *const *oms, int nprof, const msvgb_db *db,
                           double F1, void *d_xj, void *d_flags, msvgb_batch **ret_batch);
int     msvgb_batch_run(msvgb_batch *batch);
int64_t msvgb_batch_items(const msvgb_batch *batch);
int     msvgb_batch_destroy(msvgb_batch *batch);
/* Convenience: create, run once, copy the nprof * n results to host buffers, destroy. */
int     msvgb_search_batch(msvgb_ctx *ctx, const msvgb_om *const *oms, int nprof, const msvgb_db *db,
                           double F1, uint8_t *out_xj, uint8_t *out_flags);

/* ---- serving loop: continuous batching over a resident database -----------------
 * A persistent kernel consumes (request, sequence-chunk) work items that
 * submissions keep appending while it runs, so queries arriving while others
 * are on the GPU overlap with them on the device. Each request occupies one
 * device-memory slot (its cost tables, per-length tables and n-byte results);
 * the number of slots is min(max_slots, mem_budget / slot size), and
 * msvgb_server_submit blocks until a slot is free (admission by memory).
 * A request whose search fills the GPU alone (M x residues >= 40e9) runs
 * instead as its own single-query search (the tables and lane choice of
 * msvgb_profile_create), on one of two streams taken in turn; results are
 * the same either way.
 * Profiles up to M = 2047. The database must outlive the server.
 * The counterpart in the reference is the fork's per-block pipeline thread
 * (code/src/cudaHmmsearch.cu:725-810) and hmmpgmd's resident sequence cache
 * (src/hmmdwrkr.c:600-646); the calls are thread-safe. */
typedef struct msvgb_server msvgb_server;
int      msvgb_server_create(msvgb_ctx *ctx, const msvgb_db *db, double F1, int max_slots, size_t mem_budget,
                             msvgb_server **ret_server);
int      msvgb_server_slots(const msvgb_server *server);
/* Admits one query (blocking while no slot is free) and returns its ticket. */
int      msvgb_server_submit(msvgb_server *server, const msvgb_om *om, uint64_t *ret_ticket);
/* Waits (at most timeout_s seconds) for a ticket, copies its n results to
 * host buffers (either may be NULL) and frees its slot. */
int      msvgb_server_wait(msvgb_server *server, uint64_t ticket, uint8_t *out_xj, uint8_t *out_flags,
                           double timeout_s);
/* Launches of the persistent kernel, and requests run as their own searches. */
uint64_t msvgb_server_launches(const msvgb_server *server);
uint64_t msvgb_server_solo_searches(const msvgb_server *server);
int      msvgb_server_destroy(msvgb_server *server);

/* ---- pipeline driver: streamed blocks, GPU MSV stage, CPU continuation -----------
 * The threading of hmmsearch's search loop (src/hmmsearch.c:1317-1406; the
 * fork's code/src/cudaHmmsearch.cu:670-810) around the MSV stage: the calling
 * thread uploads and scores blocks of block_size sequences on the GPU, one
 * after another, while n_workers CPU threads take each scored block and call
 * fn for every sequence that passes the F1 gate, with its MSV score usc (nats,
 * +inf on overflow) -- where p7_PipelineShort (src/p7_pipeline.c:887) would
 * continue with the bias filter and the later stages. fn runs concurrently on
 * the worker threads; returning nonzero stops the run (eslFAIL). Sequences
 * are codes[off[i] .. off[i+1]) (any off[0]); *ret_n_past_msv counts passes
 * (the pipeline's n_past_msv). */
typedef int (*msvgb_survivor_fn)(void *user, int64_t seq_index, float usc, uint8_t xj, uint8_t flags);
int msvgb_pipeline_run(msvgb_ctx *ctx, const msvgb_om *om, const uint8_t *codes, const int64_t *off,
                       int64_t n, int64_t block_size, double F1, int n_workers,
                       msvgb_survivor_fn fn, void *user, int64_t *ret_n_past_msv);

/* ---- pipeline driver with the GPU filter stages after MSV ------------------------
 * The filter stages of p7_Pipeline (src/p7_pipeline.c:662-705; the fork's
 * p7_PipelineShort :887-946) on the GPU, block by block as
 * msvgb_pipeline_run streams them: the MSV stage and its F1 gate; the bias
 * filter on the MSV survivors and F1 on (usc - filtersc) (skipped when compo
 * is NULL: --nobias, filtersc = nullsc); p7_ViterbiFilter on the survivors
 * whose bias-stage P > F2 and the F2 gate on (vfsc - filtersc) with the
 * Viterbi Gumbel parameters (a sequence with P <= F2 already skips Viterbi,
 * as in the reference). fn is called on the worker threads for every
 * sequence past the Viterbi stage (past the bias stage when vom is NULL):
 * where p7_ForwardParser and domain definition would continue. */
typedef struct {
  const msvgb_om  *om;        /* MSV part; om->mmu, om->mlambda: evparam MMU, MLAMBDA */
  const msvgb_vom *vom;       /* ViterbiFilter part; NULL: stop after the bias stage  */
  const float     *compo;     /* 20 floats of model composition; NULL: no bias filter */
  float            vmu, vlambda;   /* evparam VMU, VLAMBDA                            */
  double           F1, F2;    /* 0.02 and 1e-3 by default (p7_pipeline.c:210-211)      */
} msvgb_filters;
typedef struct {
  int64_t seq_index;
  float   usc, nullsc, filtersc;
  float   vfsc;               /* NaN where Viterbi did not run (bias-stage P <= F2, or no vom) */
} msvgb_filter_hit;
typedef struct {
  int64_t nseqs, nres;
  int64_t n_past_msv, n_past_bias, n_past_vit;   /* the pipeline's counters (p7_pipeline.c:1843-1904) */
} msvgb_filter_stats;
typedef int (*msvgb_filter_fn)(void *user, const msvgb_filter_hit *hit);
int msvgb_pipeline_filters(msvgb_ctx *ctx, const msvgb_filters *f, const uint8_t *codes, const int64_t *off,
                           int64_t n, int64_t block_size, int n_workers, msvgb_filter_fn fn, void *user,
                           msvgb_filter_stats *stats);
/* A continuation that stores the hits: pass msvgb_filter_collect as fn and a
 * msvgb_filter_sink as user. Hits beyond cap are counted in n but not stored
 * (the sink never stops the run); the order is that of the worker threads. */
typedef struct {
  msvgb_filter_hit *hits;
  int64_t           cap;
  int64_t           n;        /* updated atomically */
} msvgb_filter_sink;
int msvgb_filter_collect(void *sink, const msvgb_filter_hit *hit);

/* ---- host-side score helpers (exact reference expressions) --------------------- */
/* tjb_b for target length L (p7_oprofile.c:511-519, 920-925). */
uint8_t msvgb_tjb_b(float scale_b, int L);
/* MSV score in nats from xJ (msvfilter.c:205-210); +inf when flags has ERANGE. */
float   msvgb_score(uint8_t xj, uint8_t flags, int L, uint8_t base_b, float scale_b);
/* MSV-stage gate of p7_Pipeline (p7_pipeline.c:666-676): 1 if P <= F1. */
int     msvgb_f1_pass(float usc, int L, float mmu, float mlambda, double F1, double *ret_P);

#ifdef __cplusplus
}
#endif
#endif
