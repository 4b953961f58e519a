// packed_io.cpp -- host side of makedb and of the packed/result files.
//
// makedb (src/main.cu:54-83) = check (src/makedb.hpp:59-91) + makeIndex
// (:94-156) + packData (:159-286) + groupSignatures (:289-364).  The host
// indexes the FASTA (all threads: record starts found per chunk, records
// measured in parallel), creates the packed file at its final size and writes
// its header and cleaned FASTA records into the mapped file; the device packs
// the residues of that FASTA area into bit planes, sketches and buckets them,
// and its planes and rep rows are copied into the mapped file -- every byte of
// the file is written once, and every byte is the reference's.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <thread>

#include "host.hpp"

namespace ngia {

bool InFile::open(const std::string &path) {
  fd = ::open(path.c_str(), O_RDONLY);
  if (fd < 0) return false;
  struct stat st;
  if (fstat(fd, &st) != 0) return false;
  size = (uint64_t)st.st_size;
  if (size == 0) return true;
  void *p = mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
  if (p == MAP_FAILED) return false;
  data = static_cast<const char *>(p);
  madvise(p, size, MADV_WILLNEED);
  return true;
}

void InFile::close_file() {
  if (data) munmap(const_cast<char *>(data), size);
  if (fd >= 0) ::close(fd);
  data = nullptr;
  fd = -1;
  size = 0;
}

InFile::~InFile() { close_file(); }

int OutFile::create(const std::string &path, uint64_t bytes) {
  fd = ::open(path.c_str(), O_RDWR | O_CREAT | O_TRUNC, 0644);
  if (fd < 0) return NGIA_ERR_IO;
  size = bytes;
  if (bytes == 0) return NGIA_OK;
  if (ftruncate(fd, (off_t)bytes) != 0) return NGIA_ERR_IO;
  void *p = mmap(nullptr, bytes, PROT_READ | PROT_WRITE, MAP_SHARED, fd, 0);
  if (p == MAP_FAILED) return NGIA_ERR_IO;
  data = static_cast<char *>(p);
  return NGIA_OK;
}

int OutFile::close_file() {
  bool ok = true;
  if (data) ok = munmap(data, size) == 0;
  data = nullptr;
  if (fd >= 0) ok = (::close(fd) == 0) && ok;
  fd = -1;
  return ok ? NGIA_OK : NGIA_ERR_IO;
}

OutFile::~OutFile() { close_file(); }

static unsigned worker_count() {
  unsigned t = std::thread::hardware_concurrency();
  return t ? t : 4;
}

void host_parallel_for(uint64_t n, uint64_t grain,
                       const std::function<void(uint64_t, uint64_t)> &f) {
  if (n == 0) return;
  const unsigned nt = (unsigned)std::min<uint64_t>(worker_count(), (n + grain - 1) / grain);
  if (nt <= 1) {
    f(0, n);
    return;
  }
  const uint64_t chunk = std::max<uint64_t>(grain, std::min<uint64_t>(1 << 16, n / (nt * 8) + 1));
  std::atomic<uint64_t> next(0);
  auto work = [&]() {
    for (;;) {
      const uint64_t b = next.fetch_add(chunk);
      if (b >= n) return;
      f(b, std::min(n, b + chunk));
    }
  };
  std::vector<std::thread> pool;
  for (unsigned k = 1; k < nt; ++k) pool.emplace_back(work);
  work();
  for (auto &th : pool) th.join();
}

PhaseClock::PhaseClock()
    : t0(std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch())
             .count()) {}

void PhaseClock::lap(const char *what) {
  const double t1 =
      std::chrono::duration<double>(std::chrono::steady_clock::now().time_since_epoch()).count();
  std::printf("  [%s]\t%.6f s\n", what, t1 - t0);
  t0 = t1;
}

uint32_t residue_code(unsigned char c) {
  // A reduced 15-letter alphabet shared by protein and nucleotide letters;
  // everything else codes to 0 and never matches.
  switch (c | 0x20) {
    case 'a': return 1;
    case 'c': return 2;
    case 'd': return 3;
    case 'e': case 'q': return 4;
    case 'f': case 'w': case 'y': return 5;
    case 'g': return 6;
    case 'h': return 7;
    case 'i': case 'v': return 8;
    case 'k': return 9;
    case 'l': case 'm': return 10;
    case 'n': return 11;
    case 'p': return 12;
    case 'r': return 13;
    case 's': return 14;
    case 't': case 'u': return 15;
    default: return 0;
  }
}

static int check_fasta_text(const char *d, uint64_t size, std::string &why) {
  // first line must not end with '\r'; the file must end with '\n'
  const void *nl = size ? memchr(d, '\n', size) : nullptr;
  const uint64_t eol = nl ? (uint64_t)(static_cast<const char *>(nl) - d) : size;
  if (eol > 0 && d[eol - 1] == '\r') {
    why = "Please remove the \\r at the end of lines.";
    return NGIA_ERR_FORMAT;
  }
  if (size > 0 && d[size - 1] != '\n') {
    why = "File must end with \\n.";
    return NGIA_ERR_FORMAT;
  }
  return NGIA_OK;
}

int check_fasta(const std::string &path, std::string &why) {
  InFile f;
  if (!f.open(path)) {
    why = path + " does not exist.";
    return NGIA_ERR_IO;
  }
  return check_fasta_text(f.data, f.size, why);
}

// MakeDB::makeIndex (src/makedb.hpp:94-156).  A record starts at offset 0 and
// at every line that begins with '>'; its first line is the name, the lines up
// to the next record are the read.  The record starts are found per chunk of
// the text, the records are measured in parallel, then reads of length >=
// 0xFFFF are dropped and the rest ordered by length, longest first, stably (a
// counting sort over the 65,535 possible lengths).
int make_index_text(const char *d, uint64_t n, std::vector<SeqIndex> &idx, uint64_t *scanned) {
  idx.clear();
  if (scanned) *scanned = 0;
  if (n == 0) return NGIA_OK;
  const uint64_t parts = std::max<uint64_t>(1, std::min<uint64_t>(worker_count() * 4, n >> 16));
  std::vector<std::vector<uint64_t>> found(parts);
  host_parallel_for(parts, 1, [&](uint64_t b, uint64_t e) {
    for (uint64_t k = b; k < e; ++k) {
      const uint64_t lo = n * k / parts, hi = n * (k + 1) / parts;
      std::vector<uint64_t> &f = found[k];
      if (lo == 0) f.push_back(0);
      // starts i in [lo, hi), i > 0: a newline at i - 1 in [lo - 1, hi - 1)
      uint64_t p = lo > 0 ? lo - 1 : 0;
      const uint64_t stop = hi > 0 ? hi - 1 : 0;
      while (p < stop) {
        const void *q = memchr(d + p, '\n', stop - p);
        if (!q) break;
        const uint64_t at = (uint64_t)(static_cast<const char *>(q) - d);
        if (at + 1 < n && d[at + 1] == '>') f.push_back(at + 1);
        p = at + 1;
      }
    }
  });
  std::vector<uint64_t> starts;
  size_t total = 0;
  for (auto &f : found) total += f.size();
  starts.reserve(total);
  for (auto &f : found) starts.insert(starts.end(), f.begin(), f.end());
  found.clear();
  const uint64_t R = starts.size();
  std::vector<SeqIndex> all(R);
  host_parallel_for(R, 256, [&](uint64_t b, uint64_t e) {
    for (uint64_t r = b; r < e; ++r) {
      const uint64_t s = starts[r], end = r + 1 < R ? starts[r + 1] : n;
      const void *nl = memchr(d + s, '\n', end - s);
      const uint64_t ne = nl ? (uint64_t)(static_cast<const char *>(nl) - d) : end;
      SeqIndex x;
      x.fasta_offset = s;
      x.name_len = (uint32_t)(ne - s);
      uint64_t rl = 0, rec = (ne - s) + 1;
      uint64_t pos = ne < end ? ne + 1 : end;
      while (pos < end) {  // the read's lines
        const void *q = memchr(d + pos, '\n', end - pos);
        const uint64_t qe = q ? (uint64_t)(static_cast<const char *>(q) - d) : end;
        rl += qe - pos;
        rec += (qe - pos) + 1;
        pos = qe < end ? qe + 1 : end;
      }
      x.read_len = rl > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)rl;
      x.record_bytes = rec;
      all[r] = x;
    }
  });
  if (scanned) *scanned = R;
  // stable, length descending: key 0xFFFE - len over the kept reads
  std::vector<uint32_t> count(0x10000, 0u);
  uint64_t kept = 0;
  for (const SeqIndex &x : all)
    if (x.read_len < 0xFFFF) {
      ++count[0xFFFEu - x.read_len + 1];
      ++kept;
    }
  for (size_t k = 1; k < count.size(); ++k) count[k] += count[k - 1];
  idx.resize(kept);
  for (const SeqIndex &x : all)
    if (x.read_len < 0xFFFF) idx[count[0xFFFEu - x.read_len]++] = x;
  return NGIA_OK;
}

int make_index(const std::string &path, std::vector<SeqIndex> &idx, uint64_t *scanned) {
  InFile f;
  if (!f.open(path)) return NGIA_ERR_IO;
  return make_index_text(f.data, f.size, idx, scanned);
}

int makedb_prepare(const std::string &fasta, const std::string &out, Makedb &m) {
  if (!m.in.open(fasta)) return NGIA_ERR_IO;
  std::string why;
  NGIA_TRY_HOST(check_fasta_text(m.in.data, m.in.size, why));
  std::vector<SeqIndex> idx;
  NGIA_TRY_HOST(make_index_text(m.in.data, m.in.size, idx, &m.scanned));
  if (idx.empty()) return NGIA_ERR_FORMAT;
  if (idx.size() >= 0x7FFFFFFFull) return NGIA_ERR_ARG;
  const uint32_t n = (uint32_t)idx.size();
  m.n = n;
  m.name_lens.resize(n);
  m.lens.resize(n);
  m.offsets.resize(n);
  m.text_starts.resize(n);
  std::vector<uint64_t> frel(n);  // each record's FASTA-area offset
  uint64_t words = 0, fbytes = 0;
  for (uint32_t i = 0; i < n; ++i) {
    m.name_lens[i] = idx[i].name_len;
    m.lens[i] = idx[i].read_len;
    m.offsets[i] = words;
    words += 1 + (uint64_t)((idx[i].read_len + 31u) / 32u) * 4u;
    frel[i] = fbytes;
    m.text_starts[i] = fbytes + idx[i].name_len + 1;
    fbytes += (uint64_t)idx[i].name_len + idx[i].read_len + 2;
  }
  m.words = words;
  m.pack0 = packed_area_offset(n);
  m.fasta0 = m.pack0 + words * 4;
  m.size = m.fasta0 + fbytes;
  NGIA_TRY_HOST(m.file.create(out, m.size));
  char *o = m.file.data;
  // header (src/makedb.hpp:179-197): n, name lengths, read lengths, packed and
  // FASTA offsets; the signature area and the planes come from the device
  std::memcpy(o, &n, 4);
  std::memcpy(o + 4, m.name_lens.data(), 4ull * n);
  std::memcpy(o + 4 + 4ull * n, m.lens.data(), 4ull * n);
  host_parallel_for(n, 4096, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i) {
      const uint64_t po = m.pack0 + m.offsets[i] * 4, fo = m.fasta0 + frel[i];
      std::memcpy(o + 4 + 8ull * n + 8 * i, &po, 8);
      std::memcpy(o + 4 + 16ull * n + 8 * i, &fo, 8);
    }
  });
  // cleaned FASTA records "name\nread\n" in index order (the read on one line)
  const char *src = m.in.data;
  host_parallel_for(n, 64, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i) {
      const SeqIndex &s = idx[i];
      const char *rec = src + s.fasta_offset;
      char *fo = o + m.fasta0 + frel[i];
      std::memcpy(fo, rec, s.name_len);
      fo[s.name_len] = '\n';
      char *ro = fo + s.name_len + 1;
      const char *q = rec + s.name_len + 1;
      const char *qe = rec + s.record_bytes;
      if (qe > src + m.in.size) qe = src + m.in.size;
      while (q < qe) {
        const void *nl = memchr(q, '\n', (size_t)(qe - q));
        const char *le = nl ? static_cast<const char *>(nl) : qe;
        std::memcpy(ro, q, (size_t)(le - q));
        ro += le - q;
        q = le + 1;
      }
      *ro = '\n';
    }
  });
  return NGIA_OK;
}

int makedb_finish(Makedb &m) {
  NGIA_TRY_HOST(m.file.close_file());
  m.in.close_file();
  return NGIA_OK;
}

static int check_packed_header(const InFile &f, uint32_t &n, uint64_t &words) {
  if (f.size < 4) return NGIA_ERR_FORMAT;
  std::memcpy(&n, f.data, 4);
  if (n == 0) return NGIA_ERR_FORMAT;
  const uint64_t pack0 = packed_area_offset(n);
  if (f.size < pack0) return NGIA_ERR_FORMAT;
  uint64_t p0, fasta0;
  std::memcpy(&p0, f.data + 4 + 8ull * n, 8);
  std::memcpy(&fasta0, f.data + 4 + 16ull * n, 8);
  if (p0 != pack0) return NGIA_ERR_FORMAT;
  if (fasta0 < pack0 || fasta0 > f.size || ((fasta0 - pack0) & 3u)) return NGIA_ERR_FORMAT;
  words = (fasta0 - pack0) / 4;
  return NGIA_OK;
}

// Record offsets (file bytes -> packed-area words), each record inside the
// area; rep rows below n.  All host threads.
static int check_records(const InFile &f, uint32_t n, uint64_t words, const uint32_t *lens,
                         uint32_t rep_bands, std::vector<uint64_t> &offsets) {
  const uint64_t pack0 = packed_area_offset(n), fasta0 = pack0 + 4 * words;
  offsets.resize(n);
  std::atomic<int> bad(0);
  host_parallel_for(n, 4096, [&](uint64_t b, uint64_t e) {
    bool wrong = false;
    for (uint64_t i = b; i < e; ++i) {
      uint64_t o;
      std::memcpy(&o, f.data + 4 + 8ull * n + 8 * i, 8);
      wrong |= o < pack0 || o >= fasta0 || ((o - pack0) & 3u);
      const uint64_t w = (o - pack0) / 4;
      offsets[i] = w;
      wrong |= w + 1 + (uint64_t)((lens[i] + 31u) / 32u) * 4u > words;
    }
    if (wrong) bad.store(1);
  });
  if (rep_bands) {
    const uint32_t *rep = reinterpret_cast<const uint32_t *>(f.data + sig_area_offset(n));
    host_parallel_for((uint64_t)rep_bands * n, 1 << 16, [&](uint64_t b, uint64_t e) {
      uint32_t mx = 0;
      for (uint64_t k = b; k < e; ++k) mx = std::max(mx, rep[k]);
      if (mx >= n) bad.store(1);
    });
  }
  return bad.load() ? NGIA_ERR_FORMAT : NGIA_OK;
}

int open_packed(const std::string &path, uint32_t rep_bands, PackedView &v) {
  if (!v.f.open(path)) return NGIA_ERR_IO;
  NGIA_TRY_HOST(check_packed_header(v.f, v.n, v.words));
  const uint32_t n = v.n;
  const char *d = v.f.data;
  v.name_lens = reinterpret_cast<const uint32_t *>(d + 4);
  v.lens = reinterpret_cast<const uint32_t *>(d + 4 + 4ull * n);
  v.rep = reinterpret_cast<const uint32_t *>(d + sig_area_offset(n));
  v.packed = reinterpret_cast<const uint32_t *>(d + packed_area_offset(n));
  return check_records(v.f, n, v.words, v.lens, rep_bands, v.offsets);
}

int read_packed(const std::string &path, uint32_t rep_bands, PackedDb &db) {
  PackedView v;
  NGIA_TRY_HOST(open_packed(path, rep_bands, v));
  const uint32_t n = v.n;
  db = PackedDb();
  db.n = n;
  db.name_lens.assign(v.name_lens, v.name_lens + n);
  db.lens.assign(v.lens, v.lens + n);
  db.pack_off.resize(n);
  db.fasta_off.resize(n);
  std::memcpy(db.pack_off.data(), v.f.data + 4 + 8ull * n, 8ull * n);
  std::memcpy(db.fasta_off.data(), v.f.data + 4 + 16ull * n, 8ull * n);
  db.offsets = std::move(v.offsets);
  db.packed.assign(v.packed, v.packed + v.words);
  if (rep_bands) db.rep.assign(v.rep, v.rep + (size_t)rep_bands * n);
  return NGIA_OK;
}

}  // namespace ngia

extern "C" {

int ngia_makedb(const char *fasta_path, const char *packed_path, uint32_t *n_out) {
  using namespace ngia;
  if (!fasta_path || !packed_path) return NGIA_ERR_ARG;
  if (n_out) *n_out = 0;
  Makedb m;
  NGIA_TRY_HOST(makedb_prepare(fasta_path, packed_path, m));
  ngia_ctx *ctx = nullptr;
  NGIA_TRY_HOST(ngia_ctx_create(&ctx, nullptr));
  const int st = makedb_device(ctx, m);
  ngia_ctx_destroy(ctx);
  if (st != NGIA_OK) return st;
  NGIA_TRY_HOST(makedb_finish(m));
  // size check of packData (src/makedb.hpp:271-284)
  struct stat sb;
  if (stat(packed_path, &sb) != 0 || (uint64_t)sb.st_size != m.size) return NGIA_ERR_IO;
  if (n_out) *n_out = m.n;
  return NGIA_OK;
}

// SaveResult::save (src/saveResult.hpp:31-83): clusters in ascending id, the
// representative (smallest index) as its name line and read line, every other
// member as "  " + its name line, in index order.  The line lengths are
// measured and the output laid out first, then all threads fill the mapped
// result file.
int ngia_save_result(const uint32_t *h_cluster, uint32_t n, const char *packed_path,
                     const char *result_path) {
  using namespace ngia;
  if (!h_cluster || !packed_path || !result_path || n == 0) return NGIA_ERR_ARG;
  InFile f;
  if (!f.open(packed_path) || f.size < 4) return NGIA_ERR_IO;
  uint32_t fn = 0;
  std::memcpy(&fn, f.data, 4);
  if (fn != n || f.size < packed_area_offset(n)) return NGIA_ERR_FORMAT;
  std::vector<uint64_t> fasta_off(n);
  std::memcpy(fasta_off.data(), f.data + 4 + 16ull * n, 8ull * n);
  uint32_t max_id = 0;
  for (uint32_t i = 0; i < n; ++i) max_id = std::max(max_id, h_cluster[i]);
  std::vector<uint32_t> start((size_t)max_id + 2, 0);
  for (uint32_t i = 0; i < n; ++i) start[(size_t)h_cluster[i] + 1]++;
  for (size_t c = 0; c <= max_id; ++c) start[c + 1] += start[c];
  std::vector<uint32_t> members(n), cur(start.begin(), start.end() - 1);
  for (uint32_t i = 0; i < n; ++i) members[cur[h_cluster[i]]++] = i;
  // one line of the FASTA area, without its newline
  auto line_len = [&](uint64_t off) -> uint64_t {
    if (off >= f.size) return 0;
    const void *nl = memchr(f.data + off, '\n', f.size - off);
    return (nl ? (uint64_t)(static_cast<const char *>(nl) - f.data) : f.size) - off;
  };
  std::vector<uint64_t> name_len(n), seq_len(n, 0);
  host_parallel_for(n, 1024, [&](uint64_t b, uint64_t e) {
    for (uint64_t i = b; i < e; ++i) name_len[i] = line_len(fasta_off[i]);
  });
  const uint64_t nclu = (uint64_t)max_id + 1;
  std::vector<uint64_t> at(nclu + 1, 0);  // output offset of each cluster
  host_parallel_for(nclu, 1024, [&](uint64_t b, uint64_t e) {
    for (uint64_t c = b; c < e; ++c) {
      const uint32_t lo = start[c], hi = start[c + 1];
      if (lo == hi) continue;
      const uint32_t r = members[lo];
      seq_len[r] = line_len(fasta_off[r] + name_len[r] + 1);
      uint64_t bytes = name_len[r] + 1 + seq_len[r] + 1;
      for (uint32_t k = lo + 1; k < hi; ++k) bytes += 2 + name_len[members[k]] + 1;
      at[c + 1] = bytes;
    }
  });
  for (uint64_t c = 0; c < nclu; ++c) at[c + 1] += at[c];
  OutFile out;
  NGIA_TRY_HOST(out.create(result_path, at[nclu]));
  host_parallel_for(nclu, 1024, [&](uint64_t b, uint64_t e) {
    for (uint64_t c = b; c < e; ++c) {
      const uint32_t lo = start[c], hi = start[c + 1];
      if (lo == hi) continue;
      char *o = out.data + at[c];
      const uint32_t r = members[lo];
      if (name_len[r]) std::memcpy(o, f.data + fasta_off[r], name_len[r]);
      o += name_len[r];
      *o++ = '\n';
      const uint64_t so = fasta_off[r] + name_len[r] + 1;
      if (seq_len[r]) std::memcpy(o, f.data + so, seq_len[r]);
      o += seq_len[r];
      *o++ = '\n';
      for (uint32_t k = lo + 1; k < hi; ++k) {
        const uint32_t i = members[k];
        *o++ = ' ';
        *o++ = ' ';
        if (name_len[i]) std::memcpy(o, f.data + fasta_off[i], name_len[i]);
        o += name_len[i];
        *o++ = '\n';
      }
    }
  });
  return out.close_file();
}

}  // extern "C"
