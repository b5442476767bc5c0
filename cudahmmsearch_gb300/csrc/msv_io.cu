// msv_io.cu -- the on-disk formats that feed the device.
//
//   * Pressed MSV profiles (.h3f): the first of hmmpress's four binary files,
//     one record per model as p7_oprofile_Write writes it
//     (src/impl_sse/io.c:89-120) and p7_oprofile_ReadMSV reads it
//     (io.c:233-306), HMMER 3/f format, x86-64 little-endian sizes.
//     Records hold the MSV part of a P7_OPROFILE; the reader hands it out as
//     an msvgb_om, so a pressed Pfam-style library goes straight to the
//     device. The writer produces the same record from an msvgb_om (the SSV
//     table derived from rbv as sf_conversion does, p7_oprofile.c:549-590).
//   * FASTA sequence files, digitized with Easel's amino alphabet
//     (easel/esl_alphabet.c:269-297, symbols "ACDEFGHIKLMNPQRSTVWY-BJZOUX*~",
//     case-insensitive, '_' and '.' read as '-') under the FASTA reader's
//     character map (easel/esl_sqio_ascii.c:2248-2351, inmap_fasta): blanks
//     and '\r' are skipped, '>' starts the next record, any other character is
//     an error; the name is the first word after '>' and any blanks
//     (header_fasta, esl_sqio_ascii.c:2996-3045).
//   * The packed database: the length-sorted, 16-byte-aligned residue layout
//     that msvgb_db_create builds, saved and loaded as is, so a database is
//     packed once (the job of the fork's offline dbsort tool) and later loads
//     with plain copies.
#include <algorithm>
#include <cerrno>
#include <cstdio>
#include <cstring>
#include <string>
#include <thread>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/msvgb.h"
#include "msv_internal.h"

using msvgb_detail::fail;

namespace {

// HMMER 3/f magic numbers (src/impl_sse/io.c:48-64): "3ffs" + 0x80808080 for
// the MSV file; the older formats are recognised only to name them.
constexpr uint32_t kMagic3f = 0xb3e6e6f3u;
constexpr uint32_t kOlderMagic[] = {0xb3e5e6f3u, 0xb3e4e6f3u, 0xb3e3e6f3u, 0xb3e2e6f3u, 0xe8b3e6f3u};
constexpr int kAlphaAmino = 3;           // eslAMINO (easel/esl_alphabet.h)
constexpr int kKpAmino = 29;
constexpr int kExtraSB = 17;             // p7O_EXTRA_SB (src/impl_sse/impl_sse.h:30)
constexpr int kNEvparam = 6;             // p7_NEVPARAM (src/hmmer.h:69)
constexpr int kNOffsets = 3;             // p7_NOFFSETS (src/hmmer.h:71)
constexpr int kMaxAbet = 20;             // p7_MAXABET (src/hmmer.h)
constexpr int kOffT = 8;                 // sizeof(off_t) where the file was written (LP64)

int nqb(int M) { return std::max(2, (M - 1) / 16 + 1); }   // p7O_NQB

struct Reader {
  const std::vector<uint8_t> &b;
  size_t pos = 0;
  bool ok = true;
  template <class T> T get() {
    T v{};
    if (pos + sizeof(T) > b.size()) { ok = false; return v; }
    memcpy(&v, b.data() + pos, sizeof(T));
    pos += sizeof(T);
    return v;
  }
  const uint8_t *take(size_t n) {
    if (pos + n > b.size()) { ok = false; return nullptr; }
    const uint8_t *p = b.data() + pos;
    pos += n;
    return p;
  }
};

int read_file(const char *path, std::vector<uint8_t> &out) {
  FILE *f = fopen(path, "rb");
  if (!f) return fail(MSVGB_eslENOTFOUND, std::string("cannot open ") + path + ": " + strerror(errno));
  out.clear();
  uint8_t buf[1 << 16];
  size_t k;
  while ((k = fread(buf, 1, sizeof buf, f)) > 0) out.insert(out.end(), buf, buf + k);
  const bool err = ferror(f) != 0;
  fclose(f);
  if (err) return fail(MSVGB_eslESYS, std::string("read error on ") + path);
  return MSVGB_eslOK;
}

}  // namespace

// ------------------------------------------------------------------------------
// .h3f pressed MSV profiles

struct msvgb_h3f {
  std::vector<uint8_t> data;
  size_t pos = 0;
  std::vector<uint8_t> rbv;        // the last record's table (om->rbv points here)
  float compo[20] = {};            // the last record's composition and evparam VMU, VLAMBDA
  float vmu = 0.f, vlambda = 0.f;
  bool have = false;
};

extern "C" int msvgb_h3f_open(const char *path, msvgb_h3f **ret) {
  if (!path || !ret) return fail(MSVGB_eslEINVAL, "NULL argument");
  *ret = nullptr;
  msvgb_h3f *f = new msvgb_h3f();
  int st = read_file(path, f->data);
  if (st != MSVGB_eslOK) { delete f; return st; }
  *ret = f;
  return MSVGB_eslOK;
}

extern "C" int msvgb_h3f_read(msvgb_h3f *f, msvgb_om *om, char *name, int name_cap) {
  if (!f || !om) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (f->pos >= f->data.size()) return MSVGB_eslEOF;          // no more profiles
  Reader r{f->data, f->pos};
  const uint32_t magic = r.get<uint32_t>();
  if (!r.ok) return fail(MSVGB_eslEFORMAT, "truncated record");
  for (uint32_t old : kOlderMagic)
    if (magic == old) return fail(MSVGB_eslEFORMAT, "pressed file in an older HMMER format; run hmmpress again");
  if (magic != kMagic3f) return fail(MSVGB_eslEFORMAT, "bad magic: not a HMMER 3/f MSV profile file");
  const int32_t M = r.get<int32_t>(), alpha = r.get<int32_t>(), n = r.get<int32_t>();
  if (!r.ok || M < 1 || M > 100000 || n < 0 || n > (1 << 20)) return fail(MSVGB_eslEFORMAT, "bad record header");
  const uint8_t *nm = r.take((size_t) n + 1);
  r.get<int32_t>();                                             // max_length
  const uint8_t tbm = r.get<uint8_t>(), tec = r.get<uint8_t>(), tjb = r.get<uint8_t>();
  const float scale = r.get<float>();
  const uint8_t base = r.get<uint8_t>(), bias = r.get<uint8_t>();
  if (!r.ok) return fail(MSVGB_eslEFORMAT, "truncated record");
  if (alpha != kAlphaAmino)
    return fail(MSVGB_eslEINCOMPAT, "only amino acid profiles are supported (alphabet type " + std::to_string(alpha) + ")");
  const int Q = nqb(M);
  r.take((size_t) kKpAmino * (Q + kExtraSB) * 16);              // sbv: the SSE SSV table, rebuilt on the device side
  const uint8_t *rbv = r.take((size_t) kKpAmino * Q * 16);
  float ev[kNEvparam];
  for (float &v : ev) v = r.get<float>();
  r.take((size_t) kNOffsets * kOffT);                           // hmmpfam offsets
  const uint8_t *compo = r.take((size_t) kMaxAbet * 4);
  const uint32_t tail = r.get<uint32_t>();
  if (!r.ok) return fail(MSVGB_eslEFORMAT, "truncated record");
  if (tail != kMagic3f) return fail(MSVGB_eslEFORMAT, "bad sentinel magic: corrupted .h3f record");
  f->rbv.assign(rbv, rbv + (size_t) kKpAmino * Q * 16);
  f->pos = r.pos;
  om->M = M; om->Kp = kKpAmino; om->rbv = f->rbv.data();
  om->tbm_b = tbm; om->tec_b = tec; om->tjb_b = tjb; om->base_b = base; om->bias_b = bias;
  om->scale_b = scale;
  om->mmu = ev[0]; om->mlambda = ev[1];                         // p7_MMU, p7_MLAMBDA
  memcpy(f->compo, compo, sizeof f->compo);
  f->vmu = ev[2]; f->vlambda = ev[3];                           // p7_VMU, p7_VLAMBDA
  f->have = true;
  if (name && name_cap > 0) {
    const size_t k = std::min((size_t) name_cap - 1, (size_t) n);
    memcpy(name, nm, k);
    name[k] = '\0';
  }
  return MSVGB_eslOK;
}

extern "C" int msvgb_h3f_filter_params(const msvgb_h3f *f, float *compo, float *vmu, float *vlambda) {
  if (!f || !f->have) return fail(MSVGB_eslEINVAL, "no record read yet");
  if (compo) memcpy(compo, f->compo, sizeof f->compo);
  if (vmu) *vmu = f->vmu;
  if (vlambda) *vlambda = f->vlambda;
  return MSVGB_eslOK;
}

// ------------------------------------------------------------------------------
// .h3p: the rest of a pressed profile (p7_oprofile_Write's <pfp> part,
// src/impl_sse/io.c:122-170); the ViterbiFilter fields are returned, the
// annotation and Forward/Backward fields checked for length and skipped

namespace {
constexpr uint32_t kMagic3p = 0xb3e6f0f3u;   // "3fps" + 0x80808080 (src/impl_sse/io.c:49)
constexpr int kNCutoffs = 6;                 // p7_NCUTOFFS
int nqw(int M) { return std::max(2, (M - 1) / 8 + 1); }   // p7O_NQW
int nqf(int M) { return std::max(2, (M - 1) / 4 + 1); }   // p7O_NQF
}  // namespace

struct msvgb_h3p {
  std::vector<uint8_t> data;
  size_t pos = 0;
  std::vector<int16_t> twv, rwv;   // the last record's tables (vom->twv, vom->rwv point here)
};

extern "C" int msvgb_h3p_open(const char *path, msvgb_h3p **ret) {
  if (!path || !ret) return fail(MSVGB_eslEINVAL, "NULL argument");
  *ret = nullptr;
  msvgb_h3p *f = new msvgb_h3p();
  int st = read_file(path, f->data);
  if (st != MSVGB_eslOK) { delete f; return st; }
  *ret = f;
  return MSVGB_eslOK;
}

extern "C" int msvgb_h3p_read(msvgb_h3p *f, msvgb_vom *vom, char *name, int name_cap) {
  if (!f || !vom) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (f->pos >= f->data.size()) return MSVGB_eslEOF;
  Reader r{f->data, f->pos};
  const uint32_t magic = r.get<uint32_t>();
  if (!r.ok) return fail(MSVGB_eslEFORMAT, "truncated record");
  if (magic != kMagic3p) return fail(MSVGB_eslEFORMAT, "bad magic: not a HMMER 3/f profile (.h3p) file");
  const int32_t M = r.get<int32_t>(), alpha = r.get<int32_t>(), n = r.get<int32_t>();
  if (!r.ok || M < 1 || M > 100000 || n < 0 || n > (1 << 20)) return fail(MSVGB_eslEFORMAT, "bad record header");
  if (alpha != kAlphaAmino)
    return fail(MSVGB_eslEINCOMPAT, "only amino acid profiles are supported (alphabet type " + std::to_string(alpha) + ")");
  const uint8_t *nm = r.take((size_t) n + 1);
  for (int k = 0; k < 2; ++k) {                                  // accession, description
    const int32_t len = r.get<int32_t>();
    if (!r.ok || len < 0 || len > (1 << 24)) return fail(MSVGB_eslEFORMAT, "bad accession/description length");
    if (len > 0) r.take((size_t) len + 1);
  }
  r.take((size_t) 4 * (M + 2));                                 // rf, mm, cs, consensus
  const int Q8 = nqw(M), Q4 = nqf(M);
  const uint8_t *twv = r.take((size_t) 8 * Q8 * 16);
  const uint8_t *rwv = r.take((size_t) kKpAmino * Q8 * 16);
  int16_t xw[4][2];
  for (auto &row : xw) for (int16_t &v : row) v = r.get<int16_t>();
  const float scale_w = r.get<float>();
  const int16_t base_w = r.get<int16_t>(), ddbound_w = r.get<int16_t>();
  r.get<float>();                                               // ncj_roundoff
  r.take((size_t) 8 * Q4 * 16 + (size_t) kKpAmino * Q4 * 16 + 8 * 4);   // tfv, rfv, xf: the Forward part
  r.take((size_t) kNCutoffs * 4);
  const float nj = r.get<float>();
  r.get<int32_t>(); r.get<int32_t>();                           // mode, L
  const uint32_t tail = r.get<uint32_t>();
  if (!r.ok) return fail(MSVGB_eslEFORMAT, "truncated record");
  if (tail != kMagic3p) return fail(MSVGB_eslEFORMAT, "bad sentinel magic: corrupted .h3p record");
  f->twv.resize((size_t) 8 * Q8 * 8);
  f->rwv.resize((size_t) kKpAmino * Q8 * 8);
  memcpy(f->twv.data(), twv, f->twv.size() * 2);
  memcpy(f->rwv.data(), rwv, f->rwv.size() * 2);
  f->pos = r.pos;
  vom->M = M; vom->Kp = kKpAmino;
  vom->twv = f->twv.data(); vom->rwv = f->rwv.data();
  memcpy(vom->xw, xw, sizeof xw);
  vom->scale_w = scale_w; vom->nj = nj; vom->base_w = base_w; vom->ddbound_w = ddbound_w;
  if (name && name_cap > 0) {
    const size_t k = std::min((size_t) name_cap - 1, (size_t) n);
    memcpy(name, nm, k);
    name[k] = '\0';
  }
  return MSVGB_eslOK;
}

extern "C" int msvgb_h3p_close(msvgb_h3p *f) {
  delete f;
  return MSVGB_eslOK;
}

extern "C" int msvgb_h3f_close(msvgb_h3f *f) {
  delete f;
  return MSVGB_eslOK;
}

extern "C" int msvgb_h3f_write(const char *path, const msvgb_om *om, const char *name, int append) {
  if (!path || !om || !om->rbv || !name) return fail(MSVGB_eslEINVAL, "NULL argument");
  if (om->Kp != kKpAmino || om->M < 1) return fail(MSVGB_eslEINVAL, "only amino acid profiles (Kp = 29)");
  const int M = om->M, Q = nqb(M);
  std::vector<uint8_t> b;
  auto put = [&](const void *p, size_t n) { const uint8_t *c = (const uint8_t *) p; b.insert(b.end(), c, c + n); };
  const int32_t hdr[3] = {M, kAlphaAmino, (int32_t) strlen(name)};
  const int32_t max_length = 0;
  put(&kMagic3f, 4); put(hdr, 12); put(name, strlen(name) + 1); put(&max_length, 4);
  put(&om->tbm_b, 1); put(&om->tec_b, 1); put(&om->tjb_b, 1); put(&om->scale_b, 4);
  put(&om->base_b, 1); put(&om->bias_b, 1);
  // SSV table: ((uint8_t) (bias + 127) minus rbv, unsigned saturating) ^ 127,
  // then the first p7O_EXTRA_SB vectors again (sf_conversion, p7_oprofile.c:549-590)
  const int tmp = (om->bias_b + 127) & 0xFF;
  for (int x = 0; x < kKpAmino; ++x)
    for (int q = 0; q < Q + kExtraSB; ++q)
      for (int z = 0; z < 16; ++z) {
        const int v = om->rbv[((size_t) x * Q + (q % Q)) * 16 + z];
        const uint8_t s = (uint8_t) (std::max(0, tmp - v) ^ 127);
        b.push_back(s);
      }
  put(om->rbv, (size_t) kKpAmino * Q * 16);
  const float ev[kNEvparam] = {om->mmu, om->mlambda, 0.f, 0.f, 0.f, 0.f};
  put(ev, sizeof ev);
  b.insert(b.end(), (size_t) kNOffsets * kOffT + (size_t) kMaxAbet * 4, 0);
  put(&kMagic3f, 4);
  FILE *f = fopen(path, append ? "ab" : "wb");
  if (!f) return fail(MSVGB_eslENOTFOUND, std::string("cannot write ") + path);
  const bool ok = fwrite(b.data(), 1, b.size(), f) == b.size();
  if (fclose(f) != 0 || !ok) return fail(MSVGB_eslEWRITE, std::string("write failed: ") + path);
  return MSVGB_eslOK;
}

// ------------------------------------------------------------------------------
// FASTA

struct msvgb_seqs {
  std::vector<uint8_t> codes;
  std::vector<int64_t> off{0};
  std::vector<std::string> names;
};

extern "C" int msvgb_fasta_read(const char *path, msvgb_seqs **ret) {
  if (!path || !ret) return fail(MSVGB_eslEINVAL, "NULL argument");
  *ret = nullptr;
  std::vector<uint8_t> buf;
  int st = read_file(path, buf);
  if (st != MSVGB_eslOK) return st;
  // character map: 0..28 residue codes; kSkip blanks; kEol newline; kEod '>'; kBad anything else
  enum : uint8_t { kSkip = 250, kEol = 251, kEod = 252, kBad = 255 };
  uint8_t map[256];
  memset(map, kBad, sizeof map);
  const char *sym = "ACDEFGHIKLMNPQRSTVWY-BJZOUX*~";
  for (int i = 0; i < kKpAmino; ++i) {
    map[(uint8_t) sym[i]] = (uint8_t) i;
    if (sym[i] >= 'A' && sym[i] <= 'Z') map[(uint8_t) (sym[i] - 'A' + 'a')] = (uint8_t) i;
  }
  map[(uint8_t) '_'] = map[(uint8_t) '.'] = 20;               // gap synonyms
  map[(uint8_t) ' '] = map[(uint8_t) '\t'] = map[(uint8_t) '\r'] = kSkip;
  map[(uint8_t) '\n'] = kEol;
  map[(uint8_t) '>'] = kEod;

  msvgb_seqs *s = new msvgb_seqs();
  s->codes.reserve(buf.size());
  size_t i = 0, nbuf = buf.size();
  int64_t line = 1;
  auto bad = [&](const std::string &msg) {
    delete s;
    return fail(MSVGB_eslEFORMAT, std::string(path) + " line " + std::to_string(line) + ": " + msg);
  };
  while (i < nbuf && isspace(buf[i])) { if (buf[i] == '\n') ++line; ++i; }
  while (i < nbuf) {
    if (buf[i] != '>') return bad("expected '>' at the start of a FASTA record");
    ++i;
    while (i < nbuf && (buf[i] == ' ' || buf[i] == '\t')) ++i;
    std::string name;
    while (i < nbuf && !isspace(buf[i])) name.push_back((char) buf[i++]);
    if (name.empty()) return bad("no FASTA name found");
    while (i < nbuf && buf[i] != '\n' && buf[i] != '\r') ++i;  // description: not kept
    for (; i < nbuf; ++i) {
      const uint8_t c = buf[i];
      if (c >= 128) return bad("non-ASCII character in sequence");
      const uint8_t x = map[c];
      if (x < kKpAmino) s->codes.push_back(x);
      else if (x == kEol) ++line;
      else if (x == kEod) break;
      else if (x == kBad) return bad(std::string("illegal character ") + (char) c);
    }
    s->off.push_back((int64_t) s->codes.size());
    s->names.push_back(std::move(name));
  }
  *ret = s;
  return MSVGB_eslOK;
}

extern "C" int64_t msvgb_seqs_n(const msvgb_seqs *s) { return s ? (int64_t) s->names.size() : -1; }
extern "C" const uint8_t *msvgb_seqs_codes(const msvgb_seqs *s) { return s ? s->codes.data() : nullptr; }
extern "C" const int64_t *msvgb_seqs_offsets(const msvgb_seqs *s) { return s ? s->off.data() : nullptr; }
extern "C" const char *msvgb_seqs_name(const msvgb_seqs *s, int64_t i) {
  return (s && i >= 0 && i < (int64_t) s->names.size()) ? s->names[i].c_str() : nullptr;
}
extern "C" int msvgb_seqs_free(msvgb_seqs *s) {
  delete s;
  return MSVGB_eslOK;
}

// ------------------------------------------------------------------------------
// packed database files

namespace {

const char kDbMagic[8] = {'M', 'S', 'V', 'G', 'B', 'D', 'B', '1'};

struct DbHeader {
  char magic[8];
  int64_t n, residues, packed_bytes;
};

// Checks everything a kernel will index with: lengths sorted descending and
// non-negative, 16-byte aligned starts whose padded sequences (and the 64-byte
// tail) fit in the packed buffer, padding bytes holding the padding code,
// original indices a permutation of [0, n), residue codes <= the padding code.
bool db_consistent(const DbHeader &h, const std::vector<int32_t> &len, const std::vector<int64_t> &start,
                   const std::vector<int64_t> &orig, const std::vector<uint8_t> &codes) {
  const int64_t n = h.n;
  std::vector<uint8_t> seen((size_t) n, 0);
  int64_t res = 0;
  for (int64_t s = 0; s < n; ++s) {
    if (len[s] < 0 || (s > 0 && len[s] > len[s - 1])) return false;
    const int64_t padded = ((int64_t) len[s] + 15) / 16 * 16;
    if (start[s] < 0 || (start[s] & 15) || start[s] + padded + 64 > h.packed_bytes) return false;
    for (int64_t i = start[s] + len[s]; i < start[s] + padded; ++i)   // rows past L read the padding code
      if (codes[i] != msvgb::PAD_CODE) return false;
    if (orig[s] < 0 || orig[s] >= n || seen[orig[s]]) return false;
    seen[orig[s]] = 1;
    res += len[s];
  }
  if (res != h.residues) return false;
  const int T = (int) std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
  std::vector<int> badt(T, 0);
  std::vector<std::thread> th;
  const size_t N = codes.size();
  for (int t = 0; t < T; ++t)
    th.emplace_back([&, t] {
      for (size_t i = N * t / T; i < N * (t + 1) / T; ++i)
        if (codes[i] > msvgb::PAD_CODE) { badt[t] = 1; break; }
    });
  for (auto &x : th) x.join();
  for (int b : badt) if (b) return false;
  return true;
}

}  // namespace

extern "C" int msvgb_db_save(const msvgb_db *db, const char *path) {
  if (!db || !path) return fail(MSVGB_eslEINVAL, "NULL argument");
  const int64_t n = db->n;
  std::vector<int32_t> len(n);
  std::vector<int64_t> start(n), orig(n);
  std::vector<uint8_t> codes((size_t) db->packed_bytes);
  cudaError_t e = cudaSetDevice(db->device);
  if (e == cudaSuccess && n) e = cudaMemcpy(len.data(), db->d_len, n * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n) e = cudaMemcpy(start.data(), db->d_start, n * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n) e = cudaMemcpy(orig.data(), db->d_orig, n * 8, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess) e = cudaMemcpy(codes.data(), db->d_codes, codes.size(), cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, std::string("database download: ") + cudaGetErrorString(e));
  DbHeader h;
  memcpy(h.magic, kDbMagic, 8);
  h.n = n; h.residues = db->residues; h.packed_bytes = db->packed_bytes;
  FILE *f = fopen(path, "wb");
  if (!f) return fail(MSVGB_eslENOTFOUND, std::string("cannot write ") + path);
  bool ok = fwrite(&h, sizeof h, 1, f) == 1;
  ok = ok && fwrite(len.data(), 4, n, f) == (size_t) n;
  ok = ok && fwrite(start.data(), 8, n, f) == (size_t) n;
  ok = ok && fwrite(orig.data(), 8, n, f) == (size_t) n;
  ok = ok && fwrite(codes.data(), 1, codes.size(), f) == codes.size();
  if (fclose(f) != 0 || !ok) return fail(MSVGB_eslEWRITE, std::string("write failed: ") + path);
  return MSVGB_eslOK;
}

extern "C" int msvgb_db_load(msvgb_ctx *ctx, const char *path, msvgb_db **ret) {
  if (!ctx || !path || !ret) return fail(MSVGB_eslEINVAL, "NULL argument");
  *ret = nullptr;
  FILE *f = fopen(path, "rb");
  if (!f) return fail(MSVGB_eslENOTFOUND, std::string("cannot open ") + path);
  DbHeader h;
  bool ok = fread(&h, sizeof h, 1, f) == 1 && memcmp(h.magic, kDbMagic, 8) == 0 && h.n >= 0 &&
            h.n < ((int64_t) 1 << 40) && h.residues >= 0 && h.packed_bytes >= 64 && h.packed_bytes < ((int64_t) 1 << 46);
  std::vector<int32_t> len;
  std::vector<int64_t> start, orig;
  std::vector<uint8_t> codes;
  if (ok) {
    len.resize(h.n); start.resize(h.n); orig.resize(h.n); codes.resize((size_t) h.packed_bytes);
    ok = fread(len.data(), 4, h.n, f) == (size_t) h.n && fread(start.data(), 8, h.n, f) == (size_t) h.n &&
         fread(orig.data(), 8, h.n, f) == (size_t) h.n && fread(codes.data(), 1, codes.size(), f) == codes.size();
  }
  fclose(f);
  if (!ok || !db_consistent(h, len, start, orig, codes))
    return fail(MSVGB_eslEFORMAT, std::string("not a consistent packed database file: ") + path);
  msvgb_db *db = new msvgb_db();
  db->ctx = ctx; db->device = ctx->device; db->n = h.n; db->residues = h.residues;
  db->packed_bytes = h.packed_bytes;
  db->Lmax = h.n ? len[0] : 0;
  db->serial = msvgb_detail::next_db_serial();
  for (int64_t s = h.n - 1; s >= 0; --s) {                      // ascending distinct lengths
    if (db->distinct_len.empty() || db->distinct_len.back() != len[s]) {
      db->distinct_len.push_back(len[s]);
      db->len_count.push_back(0);
    }
    db->len_count.back()++;
  }
  db->n_long = std::partition_point(len.begin(), len.end(), [](int32_t L) { return L >= kLongTarget; }) - len.begin();
  cudaError_t e = cudaSetDevice(ctx->device);
  if (e == cudaSuccess) e = cudaMalloc(&db->d_codes, codes.size());
  if (e == cudaSuccess) e = cudaMalloc(&db->d_start, std::max<int64_t>(h.n, 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&db->d_orig, std::max<int64_t>(h.n, 1) * 8);
  if (e == cudaSuccess) e = cudaMalloc(&db->d_len, std::max<int64_t>(h.n, 1) * 4);
  if (e == cudaSuccess) e = cudaMemcpy(db->d_codes, codes.data(), codes.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess && h.n) e = cudaMemcpy(db->d_start, start.data(), h.n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && h.n) e = cudaMemcpy(db->d_orig, orig.data(), h.n * 8, cudaMemcpyHostToDevice);
  if (e == cudaSuccess && h.n) e = cudaMemcpy(db->d_len, len.data(), h.n * 4, cudaMemcpyHostToDevice);
  if (e != cudaSuccess) {
    msvgb_db_destroy(db);
    return fail(e == cudaErrorMemoryAllocation ? MSVGB_eslEMEM : MSVGB_eslESYS,
                std::string("database upload: ") + cudaGetErrorString(e));
  }
  *ret = db;
  return MSVGB_eslOK;
}

extern "C" int msvgb_db_lengths(const msvgb_db *db, int32_t *out) {
  if (!db || (!out && db->n)) return fail(MSVGB_eslEINVAL, "NULL argument");
  const int64_t n = db->n;
  std::vector<int32_t> len(n);
  std::vector<int64_t> orig(n);
  cudaError_t e = cudaSetDevice(db->device);
  if (e == cudaSuccess && n) e = cudaMemcpy(len.data(), db->d_len, n * 4, cudaMemcpyDeviceToHost);
  if (e == cudaSuccess && n) e = cudaMemcpy(orig.data(), db->d_orig, n * 8, cudaMemcpyDeviceToHost);
  if (e != cudaSuccess) return fail(MSVGB_eslESYS, cudaGetErrorString(e));
  for (int64_t s = 0; s < n; ++s) out[orig[s]] = len[s];
  return MSVGB_eslOK;
}
