// host.hpp -- host-side pieces of the drop-in: packed-file I/O, makedb
// indexing and packing, Leiden, result file (internal header).
#pragma once

#include <cstdint>
#include <functional>
#include <string>
#include <vector>

#include "ngia.h"

#define NGIA_TRY_HOST(expr)       \
  do {                            \
    int s_ = (expr);              \
    if (s_ != NGIA_OK) return s_; \
  } while (0)

namespace ngia {

// The packed file (src/makedb.hpp:1-21), little-endian, no padding:
//   u32 n | u32 nameLen[n] | u32 readLen[n] | u64 packOff[n] | u64 fastaOff[n]
//   | u32 sig/rep area [64][n] | packed records | FASTA records "name\nread\n"
struct PackedDb {
  uint32_t n = 0;
  std::vector<uint32_t> name_lens, lens;
  std::vector<uint64_t> pack_off, fasta_off;  // file byte offsets
  std::vector<uint32_t> packed;               // packed record region (words)
  std::vector<uint64_t> offsets;              // word offset of each record in `packed`
  std::vector<uint32_t> rep;                  // first `bands` rep rows (band-major)
};

inline uint64_t sig_area_offset(uint64_t n) { return 4 + 24 * n; }
inline uint64_t packed_area_offset(uint64_t n) { return 4 + 24 * n + 256 * n; }

// Reads the header, offsets, `rep_bands` rep rows and the packed region.
int read_packed(const std::string &path, uint32_t rep_bands, PackedDb &db);

// One FASTA record as the index sees it (src/makedb.hpp:48-55).
struct SeqIndex {
  uint64_t fasta_offset;  // of the '>' line in the input
  uint64_t record_bytes;  // name line + sequence lines, newlines included
  uint32_t name_len;      // name line without its newline ('>' included)
  uint32_t read_len;      // residues (newlines removed)
};

// FASTA checks of MakeDB::check (src/makedb.hpp:59-91); returns 0 when ok and
// fills `why` otherwise.
int check_fasta(const std::string &path, std::string &why);

// MakeDB::makeIndex (src/makedb.hpp:94-156): records in file order, reads of
// length >= 0xFFFF dropped, then a stable sort by length descending.
int make_index(const std::string &path, std::vector<SeqIndex> &idx, uint64_t *scanned);

// The same index over text already in memory (records found and measured by
// all host threads).
int make_index_text(const char *text, uint64_t bytes, std::vector<SeqIndex> &idx,
                    uint64_t *scanned);

// A file mapped read-only.
struct InFile {
  const char *data = nullptr;
  uint64_t size = 0;
  int fd = -1;
  bool open(const std::string &path);
  void close_file();
  InFile() = default;
  InFile(const InFile &) = delete;
  InFile &operator=(const InFile &) = delete;
  ~InFile();
};

// A file created at its final size and mapped for writing: the host threads
// and the device copies write its parts in place, in any order.
struct OutFile {
  char *data = nullptr;
  uint64_t size = 0;
  int fd = -1;
  int create(const std::string &path, uint64_t bytes);
  int close_file();  // unmaps and closes; NGIA_ERR_IO if that fails
  OutFile() = default;
  OutFile(const OutFile &) = delete;
  OutFile &operator=(const OutFile &) = delete;
  ~OutFile();
};

// makedb (src/main.cu:54-83) in three steps:
//   makedb_prepare  check + index (host threads), the output file created at
//                   its final size, its header and cleaned FASTA records
//                   written (host threads);
//   makedb_device   (ctx.cu) the records' residues, read from the file's FASTA
//                   area, packed into bit planes on the device with their
//                   nibble layout, sketched and bucketed; the planes and the 64
//                   rep rows copied into the file.  The database stays loaded
//                   in the context (with its rep rows) for a graph build;
//   makedb_finish   the file closed and its size checked (src/makedb.hpp:271-284).
struct Makedb {
  InFile in;
  OutFile file;
  uint32_t n = 0;
  uint64_t scanned = 0;  // records in the FASTA, before the length filter
  uint64_t words = 0, pack0 = 0, fasta0 = 0, size = 0;
  std::vector<uint32_t> name_lens, lens;
  std::vector<uint64_t> offsets;      // word offset of each record in the packed area
  std::vector<uint64_t> text_starts;  // byte offset of its residues in the FASTA area
};
int makedb_prepare(const std::string &fasta, const std::string &out, Makedb &m);
int makedb_device(ngia_ctx *ctx, Makedb &m);
int makedb_finish(Makedb &m);

// The packed file mapped read-only: header arrays and areas in place.
struct PackedView {
  InFile f;
  uint32_t n = 0;
  uint64_t words = 0;
  const uint32_t *name_lens = nullptr, *lens = nullptr, *packed = nullptr, *rep = nullptr;
  std::vector<uint64_t> offsets;  // word offset of each record in the packed area
};
// Checks the header as read_packed does; `rep_bands` rep rows are checked
// (every entry below n).
int open_packed(const std::string &path, uint32_t rep_bands, PackedView &v);

// The `-m clustering` / `-m fast` flow (cluster.cpp).  release_device: after
// the last device step, the device is released (cudaDeviceReset) beside the
// host's Leiden and result file -- only for a process that owns the device.
int cluster_file_run(const char *packed_path, const char *result_path, uint32_t identity,
                     uint32_t bands, int fast, ngia_stats *stats, bool release_device,
                     int device);
// Graph (or fast clusters) of a loaded context -> clusters -> result file.
// Takes ctx (destroyed here); n = its record count.
int cluster_loaded(ngia_ctx *ctx, const char *packed_path, const char *result_path,
                   uint32_t identity, uint32_t bands, int fast, ngia_stats *st,
                   bool release_device, int device, uint32_t n);

// device_session.cpp: context creation and release beside host work.
void device_warmup_start(int device);
int device_warmup_join();
void device_release_start(int device);
int device_release_join();

// Calls f(begin, end) over chunks of [0, n) on all host threads.
void host_parallel_for(uint64_t n, uint64_t grain, const std::function<void(uint64_t, uint64_t)> &f);

// Phase timer of the command line's stage prints.
struct PhaseClock {
  double t0;
  PhaseClock();
  void lap(const char *what);
};

// Residue code table (src/makedb.hpp:162-171).
uint32_t residue_code(unsigned char c);

// LeidenOmp::cluster (src/leidenParallel.hpp:265-322).
std::vector<uint32_t> leiden(const std::vector<std::pair<int, int>> &edges, int n,
                             float resolution, uint64_t seed, int iterations);

}  // namespace ngia
