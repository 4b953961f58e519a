// host.hpp -- host-side pieces of the drop-in: packed-file I/O, makedb
// indexing and packing, Leiden, result file (internal header).
#pragma once

#include <cstdint>
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

// Pack every record in index order (multi-threaded on the host) and write the
// packed file with a zero signature area; returns the packed region words and
// offsets for the device stages.
int write_packed_without_sigs(const std::string &fasta, const std::string &out,
                              const std::vector<SeqIndex> &idx, PackedDb &db);

// Overwrite the signature area with the band-major rep rows (all 64 bands).
int write_rep_rows(const std::string &out, uint32_t n, const std::vector<uint32_t> &rep);

// Residue code table (src/makedb.hpp:162-171).
uint32_t residue_code(unsigned char c);

// LeidenOmp::cluster (src/leidenParallel.hpp:265-322).
std::vector<uint32_t> leiden(const std::vector<std::pair<int, int>> &edges, int n,
                             float resolution, uint64_t seed, int iterations);

}  // namespace ngia
