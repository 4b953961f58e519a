// packed_io.cpp -- host side of makedb and of the packed/result files.
//
// makedb (src/main.cu:54-83) = check (src/makedb.hpp:59-91) + makeIndex
// (:94-156) + packData (:159-286) + groupSignatures (:289-364).  Indexing and
// packing are file-bound and stay on the host (multi-threaded, the input
// mapped read-only); sketching and bucketing run on the device through the C
// ABI; the file layout and every byte of it are the reference's.
#include <fcntl.h>
#include <sys/mman.h>
#include <sys/stat.h>
#include <unistd.h>

#include <algorithm>
#include <atomic>
#include <cstdio>
#include <cstring>
#include <thread>

#include "host.hpp"

namespace ngia {

namespace {

struct MappedFile {
  const char *data = nullptr;
  size_t size = 0;
  int fd = -1;
  bool open(const std::string &path) {
    fd = ::open(path.c_str(), O_RDONLY);
    if (fd < 0) return false;
    struct stat st;
    if (fstat(fd, &st) != 0) return false;
    size = (size_t)st.st_size;
    if (size == 0) return true;
    void *p = mmap(nullptr, size, PROT_READ, MAP_PRIVATE, fd, 0);
    if (p == MAP_FAILED) return false;
    data = static_cast<const char *>(p);
    madvise(p, size, MADV_WILLNEED);
    return true;
  }
  ~MappedFile() {
    if (data) munmap(const_cast<char *>(data), size);
    if (fd >= 0) ::close(fd);
  }
};

unsigned worker_count() {
  unsigned t = std::thread::hardware_concurrency();
  return t ? t : 4;
}

template <typename F>
void parallel_for(size_t n, F &&f) {  // f(begin, end) over chunks, dynamic
  const unsigned nt = worker_count();
  const size_t chunk = std::max<size_t>(1, std::min<size_t>(4096, n / (nt * 8) + 1));
  std::atomic<size_t> next(0);
  auto work = [&]() {
    for (;;) {
      const size_t b = next.fetch_add(chunk);
      if (b >= n) return;
      f(b, std::min(n, b + chunk));
    }
  };
  std::vector<std::thread> pool;
  for (unsigned k = 1; k < nt; ++k) pool.emplace_back(work);
  work();
  for (auto &th : pool) th.join();
}

bool write_at(FILE *f, uint64_t off, const void *p, size_t bytes) {
  if (fseeko(f, (off_t)off, SEEK_SET) != 0) return false;
  return bytes == 0 || fwrite(p, 1, bytes, f) == bytes;
}

}  // namespace

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

int check_fasta(const std::string &path, std::string &why) {
  MappedFile f;
  if (!f.open(path)) {
    why = path + " does not exist.";
    return NGIA_ERR_IO;
  }
  // first line must not end with '\r'
  size_t eol = 0;
  while (eol < f.size && f.data[eol] != '\n') ++eol;
  if (eol > 0 && f.data[eol - 1] == '\r') {
    why = "Please remove the \\r at the end of lines.";
    return NGIA_ERR_FORMAT;
  }
  if (f.size > 0 && f.data[f.size - 1] != '\n') {
    why = "File must end with \\n.";
    return NGIA_ERR_FORMAT;
  }
  return NGIA_OK;
}

int make_index(const std::string &path, std::vector<SeqIndex> &idx, uint64_t *scanned) {
  MappedFile f;
  if (!f.open(path)) return NGIA_ERR_IO;
  idx.clear();
  uint64_t whole = 0;
  size_t pos = 0;
  const char *d = f.data;
  const size_t n = f.size;
  while (pos < n) {
    SeqIndex s;
    s.fasta_offset = pos;
    size_t e = pos;
    while (e < n && d[e] != '\n') ++e;
    s.name_len = (uint32_t)(e - pos);
    uint64_t rec = (e - pos) + 1;
    uint64_t rl = 0;
    pos = e < n ? e + 1 : n;
    while (pos < n && d[pos] != '>') {  // sequence lines
      size_t q = pos;
      const void *nl = memchr(d + pos, '\n', n - pos);
      q = nl ? (size_t)(static_cast<const char *>(nl) - d) : n;
      rl += q - pos;
      rec += (q - pos) + 1;
      pos = q < n ? q + 1 : n;
    }
    s.read_len = rl > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)rl;
    s.record_bytes = rec;
    ++whole;
    if (rl < 0xFFFF) idx.push_back(s);
  }
  std::stable_sort(idx.begin(), idx.end(), [](const SeqIndex &a, const SeqIndex &b) {
    return a.read_len > b.read_len;
  });
  if (scanned) *scanned = whole;
  return NGIA_OK;
}

int write_packed_without_sigs(const std::string &fasta, const std::string &out,
                              const std::vector<SeqIndex> &idx, PackedDb &db) {
  MappedFile in;
  if (!in.open(fasta)) return NGIA_ERR_IO;
  const uint32_t n = (uint32_t)idx.size();
  db = PackedDb();
  db.n = n;
  db.name_lens.resize(n);
  db.lens.resize(n);
  db.pack_off.resize(n);
  db.fasta_off.resize(n);
  db.offsets.resize(n);
  uint64_t words = 0;
  for (uint32_t i = 0; i < n; ++i) {
    db.name_lens[i] = idx[i].name_len;
    db.lens[i] = idx[i].read_len;
    db.offsets[i] = words;
    words += 1 + (uint64_t)((idx[i].read_len + 31u) / 32u) * 4u;
  }
  const uint64_t pack0 = packed_area_offset(n);
  for (uint32_t i = 0; i < n; ++i) db.pack_off[i] = pack0 + db.offsets[i] * 4;
  const uint64_t fasta0 = pack0 + words * 4;
  std::vector<uint64_t> frel(n);
  uint64_t fbytes = 0;
  for (uint32_t i = 0; i < n; ++i) {
    frel[i] = fbytes;
    db.fasta_off[i] = fasta0 + fbytes;
    fbytes += (uint64_t)idx[i].name_len + idx[i].read_len + 2;
  }
  db.packed.assign(words, 0u);
  std::vector<char> farea(fbytes);
  const char *src = in.data;
  parallel_for(n, [&](size_t b, size_t e) {
    for (size_t i = b; i < e; ++i) {
      const SeqIndex &s = idx[i];
      const char *rec = src + s.fasta_offset;
      char *fo = farea.data() + frel[i];
      std::memcpy(fo, rec, s.name_len);
      fo[s.name_len] = '\n';
      char *ro = fo + s.name_len + 1;
      uint32_t *pk = db.packed.data() + db.offsets[i];
      pk[0] = s.read_len;
      uint32_t p = 0;
      const char *q = rec + s.name_len + 1;
      const char *qe = rec + s.record_bytes;
      for (; q < qe; ++q) {
        const char ch = *q;
        if (ch == '\n') continue;
        ro[p] = ch;
        const uint32_t code = residue_code((unsigned char)ch);
        uint32_t *blk = pk + 1 + (p >> 5) * 4;
        const uint32_t bit = 1u << (p & 31u);
        if (code & 1u) blk[0] |= bit;
        if (code & 2u) blk[1] |= bit;
        if (code & 4u) blk[2] |= bit;
        if (code & 8u) blk[3] |= bit;
        ++p;
      }
      ro[p] = '\n';
    }
  });
  FILE *f = fopen(out.c_str(), "wb");
  if (!f) return NGIA_ERR_IO;
  std::vector<char> big(1 << 22);
  setvbuf(f, big.data(), _IOFBF, big.size());
  bool ok = fwrite(&n, 4, 1, f) == 1;
  ok = ok && fwrite(db.name_lens.data(), 4, n, f) == n;
  ok = ok && fwrite(db.lens.data(), 4, n, f) == n;
  ok = ok && fwrite(db.pack_off.data(), 8, n, f) == n;
  ok = ok && fwrite(db.fasta_off.data(), 8, n, f) == n;
  std::vector<uint32_t> zeros((size_t)NGIA_BANDS * n, 0u);
  ok = ok && fwrite(zeros.data(), 4, zeros.size(), f) == zeros.size();
  ok = ok && fwrite(db.packed.data(), 4, db.packed.size(), f) == db.packed.size();
  ok = ok && fwrite(farea.data(), 1, farea.size(), f) == farea.size();
  ok = (fflush(f) == 0) && ok;
  ok = (fclose(f) == 0) && ok;
  if (!ok) return NGIA_ERR_IO;
  // size check of packData (src/makedb.hpp:271-284)
  struct stat st;
  if (stat(out.c_str(), &st) != 0) return NGIA_ERR_IO;
  if ((uint64_t)st.st_size != fasta0 + fbytes) return NGIA_ERR_IO;
  return NGIA_OK;
}

int write_rep_rows(const std::string &out, uint32_t n, const std::vector<uint32_t> &rep) {
  FILE *f = fopen(out.c_str(), "r+b");
  if (!f) return NGIA_ERR_IO;
  bool ok = write_at(f, sig_area_offset(n), rep.data(), rep.size() * 4);
  ok = (fflush(f) == 0) && ok;
  ok = (fclose(f) == 0) && ok;
  return ok ? NGIA_OK : NGIA_ERR_IO;
}

int read_packed(const std::string &path, uint32_t rep_bands, PackedDb &db) {
  MappedFile f;
  if (!f.open(path)) return NGIA_ERR_IO;
  db = PackedDb();
  if (f.size < 4) return NGIA_ERR_FORMAT;
  uint32_t n = 0;
  std::memcpy(&n, f.data, 4);
  if (n == 0) return NGIA_ERR_FORMAT;
  const uint64_t pack0 = packed_area_offset(n);
  if (f.size < pack0) return NGIA_ERR_FORMAT;
  db.n = n;
  db.name_lens.resize(n);
  db.lens.resize(n);
  db.pack_off.resize(n);
  db.fasta_off.resize(n);
  const char *p = f.data + 4;
  std::memcpy(db.name_lens.data(), p, 4ull * n);
  p += 4ull * n;
  std::memcpy(db.lens.data(), p, 4ull * n);
  p += 4ull * n;
  std::memcpy(db.pack_off.data(), p, 8ull * n);
  p += 8ull * n;
  std::memcpy(db.fasta_off.data(), p, 8ull * n);
  if (db.pack_off[0] != pack0) return NGIA_ERR_FORMAT;
  const uint64_t fasta0 = db.fasta_off[0];
  if (fasta0 < pack0 || fasta0 > f.size || ((fasta0 - pack0) & 3u)) return NGIA_ERR_FORMAT;
  const uint64_t words = (fasta0 - pack0) / 4;
  db.offsets.resize(n);
  for (uint32_t i = 0; i < n; ++i) {
    const uint64_t o = db.pack_off[i];
    if (o < pack0 || o >= fasta0 || ((o - pack0) & 3u)) return NGIA_ERR_FORMAT;
    db.offsets[i] = (o - pack0) / 4;
    const uint64_t need = 1 + (uint64_t)((db.lens[i] + 31u) / 32u) * 4u;
    if (db.offsets[i] + need > words) return NGIA_ERR_FORMAT;
  }
  db.packed.resize(words);
  std::memcpy(db.packed.data(), f.data + pack0, words * 4);
  if (rep_bands) {
    db.rep.resize((size_t)rep_bands * n);
    std::memcpy(db.rep.data(), f.data + sig_area_offset(n), 4ull * rep_bands * n);
    for (uint32_t v : db.rep)
      if (v >= n) return NGIA_ERR_FORMAT;
  }
  return NGIA_OK;
}

}  // namespace ngia

extern "C" {

int ngia_makedb(const char *fasta_path, const char *packed_path, uint32_t *n_out) {
  using namespace ngia;
  if (!fasta_path || !packed_path) return NGIA_ERR_ARG;
  if (n_out) *n_out = 0;
  std::string why;
  NGIA_TRY_HOST(check_fasta(fasta_path, why));
  std::vector<SeqIndex> idx;
  uint64_t scanned = 0;
  NGIA_TRY_HOST(make_index(fasta_path, idx, &scanned));
  if (idx.empty()) return NGIA_ERR_FORMAT;
  if (idx.size() >= 0x7FFFFFFFull) return NGIA_ERR_ARG;
  PackedDb db;
  NGIA_TRY_HOST(write_packed_without_sigs(fasta_path, packed_path, idx, db));
  idx.clear();
  idx.shrink_to_fit();
  ngia_ctx *ctx = nullptr;
  NGIA_TRY_HOST(ngia_ctx_create(&ctx, nullptr));
  int st = ngia_ctx_load(ctx, db.packed.data(), db.packed.size(), db.offsets.data(),
                         db.lens.data(), db.n, nullptr, NGIA_BANDS);
  if (st == NGIA_OK) st = ngia_ctx_sketch_bucket(ctx, NGIA_BANDS);
  std::vector<uint32_t> rep;
  if (st == NGIA_OK) {
    rep.resize((size_t)NGIA_BANDS * db.n);
    st = ngia_ctx_rep_rows(ctx, rep.data(), NGIA_BANDS);
  }
  ngia_ctx_destroy(ctx);
  if (st != NGIA_OK) return st;
  NGIA_TRY_HOST(write_rep_rows(packed_path, db.n, rep));
  if (n_out) *n_out = db.n;
  return NGIA_OK;
}

int ngia_save_result(const uint32_t *h_cluster, uint32_t n, const char *packed_path,
                     const char *result_path) {
  using namespace ngia;
  if (!h_cluster || !packed_path || !result_path || n == 0) return NGIA_ERR_ARG;
  MappedFile f;
  if (!f.open(packed_path) || f.size < 4) return NGIA_ERR_IO;
  uint32_t fn = 0;
  std::memcpy(&fn, f.data, 4);
  if (fn != n || f.size < packed_area_offset(n)) return NGIA_ERR_FORMAT;
  std::vector<uint32_t> name_lens(n), lens(n);
  std::vector<uint64_t> fasta_off(n);
  std::memcpy(name_lens.data(), f.data + 4, 4ull * n);
  std::memcpy(lens.data(), f.data + 4 + 4ull * n, 4ull * n);
  std::memcpy(fasta_off.data(), f.data + 4 + 16ull * n, 8ull * n);
  // clusters in ascending id order, members in ascending index order
  uint32_t max_id = 0;
  for (uint32_t i = 0; i < n; ++i) max_id = std::max(max_id, h_cluster[i]);
  std::vector<uint32_t> start((size_t)max_id + 2, 0);
  for (uint32_t i = 0; i < n; ++i) start[(size_t)h_cluster[i] + 1]++;
  for (size_t c = 0; c <= max_id; ++c) start[c + 1] += start[c];
  std::vector<uint32_t> members(n), cur(start.begin(), start.end() - 1);
  for (uint32_t i = 0; i < n; ++i) members[cur[h_cluster[i]]++] = i;
  FILE *out = fopen(result_path, "wb");
  if (!out) return NGIA_ERR_IO;
  std::vector<char> big(1 << 22);
  setvbuf(out, big.data(), _IOFBF, big.size());
  bool ok = true;
  auto line_at = [&](uint64_t off, const char **s, size_t *len) {
    // one line of the FASTA area, without its newline
    if (off >= f.size) {
      *s = f.data + f.size;
      *len = 0;
      return;
    }
    const void *nl = memchr(f.data + off, '\n', f.size - off);
    const size_t e = nl ? (size_t)(static_cast<const char *>(nl) - f.data) : f.size;
    *s = f.data + off;
    *len = e - off;
  };
  for (size_t c = 0; c <= max_id && ok; ++c) {
    const uint32_t b = start[c], e = start[c + 1];
    if (b == e) continue;
    const uint32_t r = members[b];
    const char *s;
    size_t len;
    line_at(fasta_off[r], &s, &len);
    ok = ok && fwrite(s, 1, len, out) == len && fputc('\n', out) != EOF;
    const uint64_t seq_off = fasta_off[r] + len + 1;
    line_at(seq_off, &s, &len);
    ok = ok && fwrite(s, 1, len, out) == len && fputc('\n', out) != EOF;
    for (uint32_t k = b + 1; k < e && ok; ++k) {
      line_at(fasta_off[members[k]], &s, &len);
      ok = fputs("  ", out) != EOF && fwrite(s, 1, len, out) == len && fputc('\n', out) != EOF;
    }
  }
  ok = (fflush(out) == 0) && ok;
  ok = (fclose(out) == 0) && ok;
  return ok ? NGIA_OK : NGIA_ERR_IO;
}

}  // extern "C"
