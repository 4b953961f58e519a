// cli.cpp -- the ngia2 command line (drop-in for the reference's main,
// src/main.cu:27-164).
//
//   ngia2 -m makedb     -f <fasta>  -p <packed>
//   ngia2 -m clustering -p <packed> -r <result> [-i 95] [-b 64]
//   ngia2 -m fast       -p <packed> -r <result> [-i 95] [-b 64]
//   ngia2 cluster -i <identity> -p <packed> -r <result>   (README spelling)
//   ngia2 makeDB  -f <fasta> -p <packed>                  (README spelling)
//   ngia2 -m makedb+clustering -f <fasta> -p <packed> -r <result> [-i] [-b]
//   ngia2 -m makedb+fast       -f <fasta> -p <packed> -r <result> [-i] [-b]
// The last two run makedb and the clustering in one process (the same packed
// file and result file as the two commands), with the database kept on the
// device in between; the reference has no such mode.
//
// Flag grammar of Parser (src/parser.hpp:37-56): "-name value" pairs, the last
// occurrence wins, the final token is never read as a flag name, a missing
// required flag prints the usage.  Invalid arguments print the usage and exit
// 0; runtime failures exit 1 (src/main.cu:56-60, :88-93, :96-98).
//
// The process owns device 0 (the reference's cudaSetDevice(0)): its CUDA
// context is created on a helper thread while the host reads its input, and
// released on a helper thread while the host writes its output.
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <string>
#include <vector>

#include "host.hpp"

namespace {

struct Flag {
  const char *name;
  bool required;
  const char *help;
  std::string value;
};

// istringstream >> uint32_t as the reference's getValue does: a value that
// does not parse gives 0, which then fails the range checks.
uint32_t to_u32(const std::string &s) {
  const char *p = s.c_str();
  while (*p == ' ' || *p == '\t') ++p;
  if (*p == '\0') return 0;
  char *end = nullptr;
  const unsigned long long v = std::strtoull(p, &end, 10);
  if (end == p) return 0;
  return (uint32_t)v;
}

double since(std::chrono::steady_clock::time_point t0) {
  return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

void print_duration(const char *what, double s) {
  std::printf("%s\t%.6f s\n", what, s);
}

}  // namespace

int main(int argc, char **argv) {
  const auto t0 = std::chrono::steady_clock::now();
  std::time_t now = std::time(nullptr);
  std::printf("%s\n", std::ctime(&now));
  std::vector<Flag> flags = {
      {"-m", true, "mode (string) makedb/clustering/fast", ""},
      {"-f", false, "fasta file (string)", "data.fasta"},
      {"-p", false, "packed file (string)", "packed.bin"},
      {"-r", false, "result file (string)", "result.txt"},
      {"-i", false, "identity (1-99)", "95"},
      {"-b", false, "bands (1-64)", "64"},
  };
  // README spellings: a leading subcommand word selects the mode.
  if (argc > 1 && (std::strcmp(argv[1], "cluster") == 0 ||
                   std::strcmp(argv[1], "clustering") == 0))
    flags[0].value = "clustering";
  else if (argc > 1 && (std::strcmp(argv[1], "makeDB") == 0 ||
                        std::strcmp(argv[1], "makedb") == 0))
    flags[0].value = "makedb";
  else if (argc > 1 && std::strcmp(argv[1], "fast") == 0)
    flags[0].value = "fast";
  for (Flag &f : flags) {
    for (int i = 1; i < argc - 1; ++i)
      if (std::strcmp(argv[i], f.name) == 0) f.value = argv[i + 1];
    if (f.required && f.value.empty()) {
      std::printf("usage: %s ... (* is necessary)\n", argv[0]);
      for (const Flag &g : flags)
        if (g.required) std::printf("* %s\t%s\n", g.name, g.help);
      for (const Flag &g : flags)
        if (!g.required) std::printf("  %s\t%s\n", g.name, g.help);
      return 0;
    }
  }
  const std::string mode = flags[0].value, fasta = flags[1].value, packed = flags[2].value,
                    result = flags[3].value;
  const uint32_t identity = to_u32(flags[4].value), bands = to_u32(flags[5].value);
  int rc = 0;
  const bool both = mode == "makedb+clustering" || mode == "makedb+fast";
  if (both && (identity < 1 || identity > 99 || bands < 1 || bands > NGIA_BANDS)) {
    std::printf("identity should be 1-99, bands 1-%d\n\nUsage:\n%s -m %s -f fastaFile "
                "-p packedFile -r resultFile -i identity -b bands\n",
                NGIA_BANDS, argv[0], mode.c_str());
    return 0;
  }
  if (mode == "makedb" || both) {
    std::string why;
    if (ngia::check_fasta(fasta, why) != NGIA_OK) {
      std::printf("%s\n\nUsage:\n%s -m makedb -f fastaFile -p packedFile\n", why.c_str(),
                  argv[0]);
      return 0;
    }
    ngia::device_warmup_start(0);
    std::printf("fasta:\t%s\npacked:\t%s\n", fasta.c_str(), packed.c_str());
    ngia::PhaseClock timer;
    ngia::Makedb m;
    int st = ngia::makedb_prepare(fasta, packed, m);
    timer.lap("index + records");
    ngia_ctx *ctx = nullptr;
    if (st == NGIA_OK) st = ngia::device_warmup_join();
    if (st == NGIA_OK) st = ngia_ctx_create(&ctx, nullptr);
    timer.lap("device ready");
    if (st == NGIA_OK) st = ngia::makedb_device(ctx, m);
    timer.lap("pack + sketch + bucket");
    if (st != NGIA_OK || !both) {
      ngia_ctx_destroy(ctx);
      ngia::device_release_start(0);
    }
    if (st == NGIA_OK) st = ngia::makedb_finish(m);
    timer.lap("file");
    if (st == NGIA_ERR_FORMAT) {
      std::printf("no valid sequence (empty file or all reads >= 65535)\n");
      rc = 1;
    } else if (st != NGIA_OK) {
      std::printf("makedb failed: %s\n", ngia_status_string(st));
      rc = 1;
    } else {
      std::printf("total:\t%llu\nvalid:\t%u\n", (unsigned long long)m.scanned, m.n);
    }
    if (both && rc == 0) {
      std::printf("result file:\t%s\nidentity:\t%u\n", result.c_str(), identity);
      ngia_stats cst;
      std::memset(&cst, 0, sizeof(cst));
      const auto t1 = std::chrono::steady_clock::now();
      const bool fast = mode == "makedb+fast";
      const int s = ngia::cluster_loaded(ctx, packed.c_str(), result.c_str(), identity, bands,
                                         fast ? 1 : 0, &cst, true, 0, m.n);
      if (s != NGIA_OK) {
        std::printf("%s failed: %s\n", fast ? "fast clustering" : "clustering",
                    ngia_status_string(s));
        rc = 1;
      } else {
        print_duration(fast ? "[fast]" : "[clustering]", since(t1));
      }
    } else if (both) {
      ngia_ctx_destroy(ctx);
      ngia::device_release_start(0);
    }
    ngia::device_release_join();
  } else if (mode == "clustering" || mode == "fast") {
    const bool fast = mode == "fast";
    bool ok = true;
    FILE *pf = std::fopen(packed.c_str(), "rb");
    if (!pf) {
      std::printf("%s does not exists.\n", packed.c_str());
      ok = false;
    }
    if (identity < 1 || identity > 99) {
      std::printf("identity should be 1-99\n");
      ok = false;
    }
    if (bands < 1 || bands > NGIA_BANDS) {
      std::printf("bands should be 1-%d\n", NGIA_BANDS);
      ok = false;
    }
    if (ok && pf) {
      uint32_t n = 0;
      if (std::fread(&n, 4, 1, pf) != 1 || n == 0) {
        std::printf("%s contains 0 sequences.\n", packed.c_str());
        ok = false;
      }
    }
    if (pf) std::fclose(pf);
    if (!ok) {
      std::printf("\nUsage:\n%s -m %s -p packedFile -r resultFile -i identity -b bands\n",
                  argv[0], mode.c_str());
      return 0;
    }
    ngia::device_warmup_start(0);
    std::printf("packed file:\t%s\nresult file:\t%s\nidentity:\t%u\n", packed.c_str(),
                result.c_str(), identity);
    ngia_stats st;
    const auto t1 = std::chrono::steady_clock::now();
    const int s = ngia::cluster_file_run(packed.c_str(), result.c_str(), identity, bands,
                                         fast ? 1 : 0, &st, true, 0);
    ngia::device_release_join();
    if (s != NGIA_OK) {
      std::printf("%s failed: %s\n", fast ? "fast clustering" : "clustering",
                  ngia_status_string(s));
      rc = 1;
    } else {
      print_duration(fast ? "[fast]" : "[clustering]", since(t1));
    }
  } else {
    std::printf("Usage:\n%s -m makedb/clustering/fast\n", argv[0]);
  }
  now = std::time(nullptr);
  std::printf("\n%s", std::ctime(&now));
  print_duration("Consuming:", since(t0));
  return rc;
}
