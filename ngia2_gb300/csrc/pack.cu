// pack.cu -- device-side packing of residues into the packed-record layout
// (ngia_pack, ngia_pack_records).
//
// Restates the packing half of MakeDB::packData (src/makedb.hpp:223-231):
// each residue gets its 4-bit code from the reduced 15-letter table
// (src/makedb.hpp:162-171; case-insensitive, anything else codes to 0), and
// a record is [u32 L][4 * ceil(L/32) plane words], plane e of a 32-residue
// block holding bit e of the 32 codes.  One warp per record and block: lane j
// reads residue 32k + j (a coalesced 32-byte read), and each plane word is
// one ballot of a code bit across the warp, so the planes come out without
// any bit scatter.  Memory-bound: 1 byte read and half a byte written per
// residue.
#include <cstring>

#include "kernels.cuh"

namespace ngia {

// ASCII -> code (the table of residue_code in packed_io.cpp).
__constant__ uint8_t c_code[256];

static void code_table(uint8_t *t) {
  std::memset(t, 0, 256);
  const char *groups[15] = {"a", "c", "d", "eq", "fwy", "g", "h", "iv", "k", "lm",
                            "n", "p", "r", "s", "tu"};
  for (int g = 0; g < 15; ++g)
    for (const char *p = groups[g]; *p; ++p) {
      t[(unsigned char)*p] = (uint8_t)(g + 1);
      t[(unsigned char)(*p - 32)] = (uint8_t)(g + 1);  // upper case
    }
}

__global__ void __launch_bounds__(256)
pack_kernel(const uint8_t *__restrict__ res, const uint64_t *__restrict__ starts,
            const uint32_t *__restrict__ lens, uint32_t n, const uint64_t *__restrict__ offs,
            uint32_t *__restrict__ packed) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint32_t len = lens[i];
    const uint8_t *r = res + starts[i];
    uint32_t *pk = packed + offs[i];
    if (lane == 0) pk[0] = len;
    const uint32_t blocks = (len + 31) >> 5;
    for (uint32_t k = 0; k < blocks; ++k) {
      const uint32_t p = 32 * k + lane;
      const uint32_t code = p < len ? c_code[__ldg(r + p)] : 0u;
      const uint32_t b0 = __ballot_sync(kFull, code & 1u), b1 = __ballot_sync(kFull, code & 2u);
      const uint32_t b2 = __ballot_sync(kFull, code & 4u), b3 = __ballot_sync(kFull, code & 8u);
      if (lane < 4) pk[1 + 4 * k + lane] = lane == 0 ? b0 : lane == 1 ? b1 : lane == 2 ? b2 : b3;
    }
  }
}

// The same packing, plus the nibble layout the sketch and the aligners read
// (word q of a block: residues 8q..8q+7, the first in the high nibble; the
// length word copied) and the set of residue codes present, in one pass: a
// database loaded from residue text (makedb) never reads its planes back.
// Lane j's code shifted to its nibble and OR-ed across each group of eight
// lanes gives nibble word j / 8 in lanes 0, 8, 16, 24.
__global__ void __launch_bounds__(256)
pack_layout_kernel(const uint8_t *__restrict__ res, const uint64_t *__restrict__ starts,
                   const uint32_t *__restrict__ lens, uint32_t n,
                   const uint64_t *__restrict__ offs, uint32_t *__restrict__ packed,
                   uint32_t *__restrict__ nib, uint32_t *__restrict__ presence) {
  const uint32_t lane = threadIdx.x & 31u;
  const uint32_t warps = (gridDim.x * blockDim.x) >> 5;
  uint32_t mine = 0;
  for (uint32_t i = (blockIdx.x * blockDim.x + threadIdx.x) >> 5; i < n; i += warps) {
    const uint32_t len = lens[i];
    const uint8_t *r = res + starts[i];
    const uint64_t o = offs[i];
    if (lane == 0) {
      packed[o] = len;
      nib[o] = len;
    }
    const uint32_t blocks = (len + 31) >> 5;
    for (uint32_t k = 0; k < blocks; ++k) {
      const uint32_t p = 32 * k + lane;
      const bool real = p < len;
      const uint32_t code = real ? c_code[__ldg(r + p)] : 0u;
      if (real) mine |= 1u << code;
      const uint32_t b0 = __ballot_sync(kFull, code & 1u), b1 = __ballot_sync(kFull, code & 2u);
      const uint32_t b2 = __ballot_sync(kFull, code & 4u), b3 = __ballot_sync(kFull, code & 8u);
      uint32_t x = code << (4u * (7u - (lane & 7u)));
      x |= __shfl_xor_sync(kFull, x, 1);
      x |= __shfl_xor_sync(kFull, x, 2);
      x |= __shfl_xor_sync(kFull, x, 4);
      const uint64_t blk = o + 1 + 4ull * k;
      if (lane < 4) packed[blk + lane] = lane == 0 ? b0 : lane == 1 ? b1 : lane == 2 ? b2 : b3;
      if ((lane & 7u) == 0) nib[blk + (lane >> 3)] = x;
    }
  }
  mine = __reduce_or_sync(kFull, mine);
  if (lane == 0 && mine) atomicOr(presence, mine);
}

static int upload_table() {
  static bool done[64] = {};
  int dev = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  if (dev >= 0 && dev < 64 && done[dev]) return NGIA_OK;
  uint8_t t[256];
  code_table(t);
  NGIA_CUDA(cudaMemcpyToSymbol(c_code, t, sizeof(t)));
  if (dev >= 0 && dev < 64) done[dev] = true;
  return NGIA_OK;
}

int launch_pack(const uint8_t *res, const uint64_t *starts, const uint32_t *lens, uint32_t n,
                const uint64_t *offs, uint32_t *packed, cudaStream_t s) {
  if (n == 0) return NGIA_OK;
  NGIA_TRY(upload_table());
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t want = ceil_div(n, 8u), cap = (uint32_t)sms * 16u;
  pack_kernel<<<want < cap ? want : cap, 256, 0, s>>>(res, starts, lens, n, offs, packed);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

int launch_pack_layout(const uint8_t *res, const uint64_t *starts, const uint32_t *lens,
                       uint32_t n, const uint64_t *offs, uint32_t *packed, uint32_t *nib,
                       uint32_t *presence, cudaStream_t s) {
  NGIA_CUDA(cudaMemsetAsync(presence, 0, sizeof(uint32_t), s));
  if (n == 0) return NGIA_OK;
  NGIA_TRY(upload_table());
  int dev = 0, sms = 0;
  NGIA_CUDA(cudaGetDevice(&dev));
  NGIA_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
  const uint32_t want = ceil_div(n, 8u), cap = (uint32_t)sms * 16u;
  pack_layout_kernel<<<want < cap ? want : cap, 256, 0, s>>>(res, starts, lens, n, offs, packed,
                                                             nib, presence);
  NGIA_LAUNCHED();
  return NGIA_OK;
}

}  // namespace ngia

extern "C" {

int ngia_pack(const uint8_t *d_residues, const uint64_t *d_starts, const uint32_t *d_lens,
              uint32_t n, const uint64_t *d_rec_offsets, uint32_t *d_packed, void *stream) {
  if (n == 0) return NGIA_OK;
  if (!d_residues || !d_starts || !d_lens || !d_rec_offsets || !d_packed) return NGIA_ERR_ARG;
  return ngia::launch_pack(d_residues, d_starts, d_lens, n, d_rec_offsets, d_packed,
                           ngia::as_stream(stream));
}

int ngia_pack_records(const uint8_t *h_residues, uint64_t residue_bytes,
                      const uint64_t *h_starts, const uint32_t *h_lens, uint32_t n,
                      uint32_t *h_packed, uint64_t words, uint64_t *h_rec_offsets) {
  if (n == 0) return NGIA_OK;
  if (!h_residues || !h_starts || !h_lens || !h_packed || !h_rec_offsets) return NGIA_ERR_ARG;
  uint64_t w = 0;
  for (uint32_t i = 0; i < n; ++i) {  // records back to back, checked against the inputs
    if (h_lens[i] > NGIA_MAX_READ || h_starts[i] + h_lens[i] > residue_bytes) return NGIA_ERR_ARG;
    h_rec_offsets[i] = w;
    w += 1 + 4ull * ((h_lens[i] + 31) / 32);
  }
  if (w > words) return NGIA_ERR_ARG;
  uint8_t *d_res = nullptr;
  uint64_t *d_starts = nullptr, *d_offs = nullptr;
  uint32_t *d_lens = nullptr, *d_packed = nullptr;
  int rc = NGIA_OK;
  auto check = [&](cudaError_t e) {
    if (rc == NGIA_OK && e != cudaSuccess) rc = ngia::cuda_fail(e);
  };
  check(cudaMalloc(&d_res, residue_bytes ? residue_bytes : 1));
  check(cudaMalloc(&d_starts, (size_t)n * 8));
  check(cudaMalloc(&d_offs, (size_t)n * 8));
  check(cudaMalloc(&d_lens, (size_t)n * 4));
  check(cudaMalloc(&d_packed, w * 4));
  if (rc == NGIA_OK) {
    check(cudaMemcpy(d_res, h_residues, residue_bytes, cudaMemcpyHostToDevice));
    check(cudaMemcpy(d_starts, h_starts, (size_t)n * 8, cudaMemcpyHostToDevice));
    check(cudaMemcpy(d_offs, h_rec_offsets, (size_t)n * 8, cudaMemcpyHostToDevice));
    check(cudaMemcpy(d_lens, h_lens, (size_t)n * 4, cudaMemcpyHostToDevice));
  }
  if (rc == NGIA_OK) rc = ngia::launch_pack(d_res, d_starts, d_lens, n, d_offs, d_packed, 0);
  if (rc == NGIA_OK) check(cudaMemcpy(h_packed, d_packed, w * 4, cudaMemcpyDeviceToHost));
  cudaFree(d_res);
  cudaFree(d_starts);
  cudaFree(d_offs);
  cudaFree(d_lens);
  cudaFree(d_packed);
  return rc;
}

}  // extern "C"
