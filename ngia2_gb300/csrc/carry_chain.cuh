// carry_chain.cuh -- multi-word add-with-carry chains in inline PTX
// (internal header).
//
// add_chainN_XY(s, a, b[, cin][, cout]) computes the N-word sum
//   s[0..N) = a[0..N) + b[0..N) + carry_in
// with the carry rippling from word 0 upward through the hardware carry flag
// (add.cc / addc.cc), one instruction per word.
//   X = z : carry_in = 0
//   X = c : carry_in = (cin != 0) (cin + 0xFFFFFFFF sets the flag)
//   Y = n : no carry out
//   Y = c : cout = carry out of word N-1 (0 or 1)
#pragma once
#include <cstdint>

namespace ngia {

__device__ __forceinline__ void add_chain2_zn(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm("add.cc.u32 %0, %2, %4;\n\t"
      "addc.u32 %1, %3, %5;\n\t"
      : "=r"(s[0]), "=r"(s[1])
      : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void add_chain2_zc(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t &cout) {
  asm("add.cc.u32 %0, %3, %5;\n\t"
      "addc.cc.u32 %1, %4, %6;\n\t"
      "addc.u32 %2, 0, 0;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void add_chain2_cn(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t cin) {
  asm("{\n\t.reg .u32 t;\n\t"
      "add.cc.u32 t, %6, 0xFFFFFFFF;\n\t"
      "addc.cc.u32 %0, %2, %4;\n\t"
      "addc.u32 %1, %3, %5;\n\t"
      "}"
      : "=r"(s[0]), "=r"(s[1])
      : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]), "r"(cin));
}

__device__ __forceinline__ void add_chain2_cc(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t cin, uint32_t &cout) {
  asm("{\n\t.reg .u32 t;\n\t"
      "add.cc.u32 t, %7, 0xFFFFFFFF;\n\t"
      "addc.cc.u32 %0, %3, %5;\n\t"
      "addc.cc.u32 %1, %4, %6;\n\t"
      "addc.u32 %2, 0, 0;\n\t"
      "}"
      : "=r"(s[0]), "=r"(s[1]), "=r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]), "r"(cin));
}

__device__ __forceinline__ void add_chain4_zn(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm("add.cc.u32 %0, %4, %8;\n\t"
      "addc.cc.u32 %1, %5, %9;\n\t"
      "addc.cc.u32 %2, %6, %10;\n\t"
      "addc.u32 %3, %7, %11;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
}

__device__ __forceinline__ void add_chain4_zc(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t &cout) {
  asm("add.cc.u32 %0, %5, %9;\n\t"
      "addc.cc.u32 %1, %6, %10;\n\t"
      "addc.cc.u32 %2, %7, %11;\n\t"
      "addc.cc.u32 %3, %8, %12;\n\t"
      "addc.u32 %4, 0, 0;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
}

__device__ __forceinline__ void add_chain4_cn(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t cin) {
  asm("{\n\t.reg .u32 t;\n\t"
      "add.cc.u32 t, %12, 0xFFFFFFFF;\n\t"
      "addc.cc.u32 %0, %4, %8;\n\t"
      "addc.cc.u32 %1, %5, %9;\n\t"
      "addc.cc.u32 %2, %6, %10;\n\t"
      "addc.u32 %3, %7, %11;\n\t"
      "}"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(cin));
}

__device__ __forceinline__ void add_chain4_cc(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t cin, uint32_t &cout) {
  asm("{\n\t.reg .u32 t;\n\t"
      "add.cc.u32 t, %13, 0xFFFFFFFF;\n\t"
      "addc.cc.u32 %0, %5, %9;\n\t"
      "addc.cc.u32 %1, %6, %10;\n\t"
      "addc.cc.u32 %2, %7, %11;\n\t"
      "addc.cc.u32 %3, %8, %12;\n\t"
      "addc.u32 %4, 0, 0;\n\t"
      "}"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(cin));
}

__device__ __forceinline__ void add_chain8_zn(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm("add.cc.u32 %0, %8, %16;\n\t"
      "addc.cc.u32 %1, %9, %17;\n\t"
      "addc.cc.u32 %2, %10, %18;\n\t"
      "addc.cc.u32 %3, %11, %19;\n\t"
      "addc.cc.u32 %4, %12, %20;\n\t"
      "addc.cc.u32 %5, %13, %21;\n\t"
      "addc.cc.u32 %6, %14, %22;\n\t"
      "addc.u32 %7, %15, %23;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

__device__ __forceinline__ void add_chain8_zc(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t &cout) {
  asm("add.cc.u32 %0, %9, %17;\n\t"
      "addc.cc.u32 %1, %10, %18;\n\t"
      "addc.cc.u32 %2, %11, %19;\n\t"
      "addc.cc.u32 %3, %12, %20;\n\t"
      "addc.cc.u32 %4, %13, %21;\n\t"
      "addc.cc.u32 %5, %14, %22;\n\t"
      "addc.cc.u32 %6, %15, %23;\n\t"
      "addc.cc.u32 %7, %16, %24;\n\t"
      "addc.u32 %8, 0, 0;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

__device__ __forceinline__ void add_chain8_cn(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t cin) {
  asm("{\n\t.reg .u32 t;\n\t"
      "add.cc.u32 t, %24, 0xFFFFFFFF;\n\t"
      "addc.cc.u32 %0, %8, %16;\n\t"
      "addc.cc.u32 %1, %9, %17;\n\t"
      "addc.cc.u32 %2, %10, %18;\n\t"
      "addc.cc.u32 %3, %11, %19;\n\t"
      "addc.cc.u32 %4, %12, %20;\n\t"
      "addc.cc.u32 %5, %13, %21;\n\t"
      "addc.cc.u32 %6, %14, %22;\n\t"
      "addc.u32 %7, %15, %23;\n\t"
      "}"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(cin));
}

__device__ __forceinline__ void add_chain8_cc(uint32_t *s, const uint32_t *a, const uint32_t *b, uint32_t cin, uint32_t &cout) {
  asm("{\n\t.reg .u32 t;\n\t"
      "add.cc.u32 t, %25, 0xFFFFFFFF;\n\t"
      "addc.cc.u32 %0, %9, %17;\n\t"
      "addc.cc.u32 %1, %10, %18;\n\t"
      "addc.cc.u32 %2, %11, %19;\n\t"
      "addc.cc.u32 %3, %12, %20;\n\t"
      "addc.cc.u32 %4, %13, %21;\n\t"
      "addc.cc.u32 %5, %14, %22;\n\t"
      "addc.cc.u32 %6, %15, %23;\n\t"
      "addc.cc.u32 %7, %16, %24;\n\t"
      "addc.u32 %8, 0, 0;\n\t"
      "}"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(cin));
}

// ---- carry words ---------------------------------------------------------------
// Chains whose carry in is popped from the top bit of a word (add.cc x, x, x:
// the flag takes bit 31, x shifts left) and whose carry out is appended at
// the bottom of another (addc x, x, x: x = 2x + flag).  32 calls in column
// order fill `cout` with column 0's carry in bit 31, which is the order the
// next chain pops them in.
//   add_chainN_pp : pop in, push out
//   add_chain8_pc : pop in, carry out as 0/1 in c (first half of 16 words)
//   add_chain8_cp : carry in from c != 0, push out (second half)
__device__ __forceinline__ void add_chain1_pp(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                              uint32_t &cin, uint32_t &cout) {
  asm("add.cc.u32 %1, %1, %1;\n\t"
      "addc.cc.u32 %0, %3, %4;\n\t"
      "addc.u32 %2, %2, %2;\n\t"
      : "=r"(s[0]), "+r"(cin), "+r"(cout)
      : "r"(a[0]), "r"(b[0]));
}

__device__ __forceinline__ void add_chain2_pp(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                              uint32_t &cin, uint32_t &cout) {
  asm("add.cc.u32 %2, %2, %2;\n\t"
      "addc.cc.u32 %0, %4, %6;\n\t"
      "addc.cc.u32 %1, %5, %7;\n\t"
      "addc.u32 %3, %3, %3;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "+r"(cin), "+r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]));
}

__device__ __forceinline__ void add_chain4_pp(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                              uint32_t &cin, uint32_t &cout) {
  asm("add.cc.u32 %4, %4, %4;\n\t"
      "addc.cc.u32 %0, %6, %10;\n\t"
      "addc.cc.u32 %1, %7, %11;\n\t"
      "addc.cc.u32 %2, %8, %12;\n\t"
      "addc.cc.u32 %3, %9, %13;\n\t"
      "addc.u32 %5, %5, %5;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "+r"(cin), "+r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
}

__device__ __forceinline__ void add_chain8_pp(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                              uint32_t &cin, uint32_t &cout) {
  asm("add.cc.u32 %8, %8, %8;\n\t"
      "addc.cc.u32 %0, %10, %18;\n\t"
      "addc.cc.u32 %1, %11, %19;\n\t"
      "addc.cc.u32 %2, %12, %20;\n\t"
      "addc.cc.u32 %3, %13, %21;\n\t"
      "addc.cc.u32 %4, %14, %22;\n\t"
      "addc.cc.u32 %5, %15, %23;\n\t"
      "addc.cc.u32 %6, %16, %24;\n\t"
      "addc.cc.u32 %7, %17, %25;\n\t"
      "addc.u32 %9, %9, %9;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "+r"(cin), "+r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

__device__ __forceinline__ void add_chain8_pc(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                              uint32_t &cin, uint32_t &c) {
  asm("add.cc.u32 %8, %8, %8;\n\t"
      "addc.cc.u32 %0, %10, %18;\n\t"
      "addc.cc.u32 %1, %11, %19;\n\t"
      "addc.cc.u32 %2, %12, %20;\n\t"
      "addc.cc.u32 %3, %13, %21;\n\t"
      "addc.cc.u32 %4, %14, %22;\n\t"
      "addc.cc.u32 %5, %15, %23;\n\t"
      "addc.cc.u32 %6, %16, %24;\n\t"
      "addc.cc.u32 %7, %17, %25;\n\t"
      "addc.u32 %9, 0, 0;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "+r"(cin), "=r"(c)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]));
}

__device__ __forceinline__ void add_chain8_cp(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                              uint32_t c, uint32_t &cout) {
  asm("{\n\t.reg .u32 t;\n\t"
      "add.cc.u32 t, %25, 0xFFFFFFFF;\n\t"
      "addc.cc.u32 %0, %9, %17;\n\t"
      "addc.cc.u32 %1, %10, %18;\n\t"
      "addc.cc.u32 %2, %11, %19;\n\t"
      "addc.cc.u32 %3, %12, %20;\n\t"
      "addc.cc.u32 %4, %13, %21;\n\t"
      "addc.cc.u32 %5, %14, %22;\n\t"
      "addc.cc.u32 %6, %15, %23;\n\t"
      "addc.cc.u32 %7, %16, %24;\n\t"
      "addc.u32 %8, %8, %8;\n\t"
      "}"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "+r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(c));
}

// s[0..K) = a + b + (carry popped from cin), carry out pushed into cout.
template <int K>
__device__ __forceinline__ void add_words_pp(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                             uint32_t &cin, uint32_t &cout) {
  if constexpr (K == 1) add_chain1_pp(s, a, b, cin, cout);
  else if constexpr (K == 2) add_chain2_pp(s, a, b, cin, cout);
  else if constexpr (K == 4) add_chain4_pp(s, a, b, cin, cout);
  else if constexpr (K == 8) add_chain8_pp(s, a, b, cin, cout);
  else {
    static_assert(K == 16, "carry-word chains of 1, 2, 4, 8 or 16 words");
    uint32_t c;
    add_chain8_pc(s, a, b, cin, c);
    add_chain8_cp(s + 8, a + 8, b + 8, c, cout);
  }
}

}  // namespace ngia
