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

__device__ __forceinline__ void add_chain3_pp(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                              uint32_t &cin, uint32_t &cout) {
  asm("add.cc.u32 %3, %3, %3;\n\t"
      "addc.cc.u32 %0, %5, %8;\n\t"
      "addc.cc.u32 %1, %6, %9;\n\t"
      "addc.cc.u32 %2, %7, %10;\n\t"
      "addc.u32 %4, %4, %4;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "+r"(cin), "+r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(b[0]), "r"(b[1]), "r"(b[2]));
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

__device__ __forceinline__ void add_chain6_pp(uint32_t *s, const uint32_t *a, const uint32_t *b,
                                              uint32_t &cin, uint32_t &cout) {
  asm("add.cc.u32 %6, %6, %6;\n\t"
      "addc.cc.u32 %0, %8, %14;\n\t"
      "addc.cc.u32 %1, %9, %15;\n\t"
      "addc.cc.u32 %2, %10, %16;\n\t"
      "addc.cc.u32 %3, %11, %17;\n\t"
      "addc.cc.u32 %4, %12, %18;\n\t"
      "addc.cc.u32 %5, %13, %19;\n\t"
      "addc.u32 %7, %7, %7;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "+r"(cin), "+r"(cout)
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]),
        "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]));
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
  else if constexpr (K == 3) add_chain3_pp(s, a, b, cin, cout);
  else if constexpr (K == 4) add_chain4_pp(s, a, b, cin, cout);
  else if constexpr (K == 6) add_chain6_pp(s, a, b, cin, cout);
  else if constexpr (K == 8) add_chain8_pp(s, a, b, cin, cout);
  else {
    static_assert(K == 16, "carry-word chains of 1, 2, 3, 4, 6, 8 or 16 words");
    uint32_t c;
    add_chain8_pc(s, a, b, cin, c);
    add_chain8_cp(s + 8, a + 8, b + 8, c, cout);
  }
}


// ---- one chain of any length 1..16, no carry in or out -------------------------
// add_run<N>(s, a, b): s[0..N) = a[0..N) + b[0..N) as one N-word number, the
// carry rippling through the flag across the whole run (no carry value
// materialised between words).  Written out for each N.
__device__ __forceinline__ void add_run1(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.u32 %0, %1, %2;\n\t"
      : "=r"(s[0])
      : "r"(a[0]), "r"(b[0]));
}
__device__ __forceinline__ void add_run2(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %2, %4;\n\t"
      "addc.u32 %1, %3, %5;\n\t"
      : "=r"(s[0]), "=r"(s[1])
      : "r"(a[0]), "r"(a[1]), "r"(b[0]), "r"(b[1]));
}
__device__ __forceinline__ void add_run3(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %3, %6;\n\t"
      "addc.cc.u32 %1, %4, %7;\n\t"
      "addc.u32 %2, %5, %8;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(b[0]), "r"(b[1]), "r"(b[2]));
}
__device__ __forceinline__ void add_run4(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %4, %8;\n\t"
      "addc.cc.u32 %1, %5, %9;\n\t"
      "addc.cc.u32 %2, %6, %10;\n\t"
      "addc.u32 %3, %7, %11;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]));
}
__device__ __forceinline__ void add_run5(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %5, %10;\n\t"
      "addc.cc.u32 %1, %6, %11;\n\t"
      "addc.cc.u32 %2, %7, %12;\n\t"
      "addc.cc.u32 %3, %8, %13;\n\t"
      "addc.u32 %4, %9, %14;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]));
}
__device__ __forceinline__ void add_run6(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %6, %12;\n\t"
      "addc.cc.u32 %1, %7, %13;\n\t"
      "addc.cc.u32 %2, %8, %14;\n\t"
      "addc.cc.u32 %3, %9, %15;\n\t"
      "addc.cc.u32 %4, %10, %16;\n\t"
      "addc.u32 %5, %11, %17;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]));
}
__device__ __forceinline__ void add_run7(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %7, %14;\n\t"
      "addc.cc.u32 %1, %8, %15;\n\t"
      "addc.cc.u32 %2, %9, %16;\n\t"
      "addc.cc.u32 %3, %10, %17;\n\t"
      "addc.cc.u32 %4, %11, %18;\n\t"
      "addc.cc.u32 %5, %12, %19;\n\t"
      "addc.u32 %6, %13, %20;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]));
}
__device__ __forceinline__ void add_run8(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %8, %16;\n\t"
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
__device__ __forceinline__ void add_run9(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %9, %18;\n\t"
      "addc.cc.u32 %1, %10, %19;\n\t"
      "addc.cc.u32 %2, %11, %20;\n\t"
      "addc.cc.u32 %3, %12, %21;\n\t"
      "addc.cc.u32 %4, %13, %22;\n\t"
      "addc.cc.u32 %5, %14, %23;\n\t"
      "addc.cc.u32 %6, %15, %24;\n\t"
      "addc.cc.u32 %7, %16, %25;\n\t"
      "addc.u32 %8, %17, %26;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]));
}
__device__ __forceinline__ void add_run10(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %10, %20;\n\t"
      "addc.cc.u32 %1, %11, %21;\n\t"
      "addc.cc.u32 %2, %12, %22;\n\t"
      "addc.cc.u32 %3, %13, %23;\n\t"
      "addc.cc.u32 %4, %14, %24;\n\t"
      "addc.cc.u32 %5, %15, %25;\n\t"
      "addc.cc.u32 %6, %16, %26;\n\t"
      "addc.cc.u32 %7, %17, %27;\n\t"
      "addc.cc.u32 %8, %18, %28;\n\t"
      "addc.u32 %9, %19, %29;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]));
}
__device__ __forceinline__ void add_run11(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %11, %22;\n\t"
      "addc.cc.u32 %1, %12, %23;\n\t"
      "addc.cc.u32 %2, %13, %24;\n\t"
      "addc.cc.u32 %3, %14, %25;\n\t"
      "addc.cc.u32 %4, %15, %26;\n\t"
      "addc.cc.u32 %5, %16, %27;\n\t"
      "addc.cc.u32 %6, %17, %28;\n\t"
      "addc.cc.u32 %7, %18, %29;\n\t"
      "addc.cc.u32 %8, %19, %30;\n\t"
      "addc.cc.u32 %9, %20, %31;\n\t"
      "addc.u32 %10, %21, %32;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]));
}
__device__ __forceinline__ void add_run12(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %12, %24;\n\t"
      "addc.cc.u32 %1, %13, %25;\n\t"
      "addc.cc.u32 %2, %14, %26;\n\t"
      "addc.cc.u32 %3, %15, %27;\n\t"
      "addc.cc.u32 %4, %16, %28;\n\t"
      "addc.cc.u32 %5, %17, %29;\n\t"
      "addc.cc.u32 %6, %18, %30;\n\t"
      "addc.cc.u32 %7, %19, %31;\n\t"
      "addc.cc.u32 %8, %20, %32;\n\t"
      "addc.cc.u32 %9, %21, %33;\n\t"
      "addc.cc.u32 %10, %22, %34;\n\t"
      "addc.u32 %11, %23, %35;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]));
}
__device__ __forceinline__ void add_run13(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %13, %26;\n\t"
      "addc.cc.u32 %1, %14, %27;\n\t"
      "addc.cc.u32 %2, %15, %28;\n\t"
      "addc.cc.u32 %3, %16, %29;\n\t"
      "addc.cc.u32 %4, %17, %30;\n\t"
      "addc.cc.u32 %5, %18, %31;\n\t"
      "addc.cc.u32 %6, %19, %32;\n\t"
      "addc.cc.u32 %7, %20, %33;\n\t"
      "addc.cc.u32 %8, %21, %34;\n\t"
      "addc.cc.u32 %9, %22, %35;\n\t"
      "addc.cc.u32 %10, %23, %36;\n\t"
      "addc.cc.u32 %11, %24, %37;\n\t"
      "addc.u32 %12, %25, %38;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11]), "=r"(s[12])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(a[12]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]), "r"(b[12]));
}
__device__ __forceinline__ void add_run14(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %14, %28;\n\t"
      "addc.cc.u32 %1, %15, %29;\n\t"
      "addc.cc.u32 %2, %16, %30;\n\t"
      "addc.cc.u32 %3, %17, %31;\n\t"
      "addc.cc.u32 %4, %18, %32;\n\t"
      "addc.cc.u32 %5, %19, %33;\n\t"
      "addc.cc.u32 %6, %20, %34;\n\t"
      "addc.cc.u32 %7, %21, %35;\n\t"
      "addc.cc.u32 %8, %22, %36;\n\t"
      "addc.cc.u32 %9, %23, %37;\n\t"
      "addc.cc.u32 %10, %24, %38;\n\t"
      "addc.cc.u32 %11, %25, %39;\n\t"
      "addc.cc.u32 %12, %26, %40;\n\t"
      "addc.u32 %13, %27, %41;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11]), "=r"(s[12]), "=r"(s[13])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(a[12]), "r"(a[13]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]), "r"(b[12]), "r"(b[13]));
}
__device__ __forceinline__ void add_run15(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %15, %30;\n\t"
      "addc.cc.u32 %1, %16, %31;\n\t"
      "addc.cc.u32 %2, %17, %32;\n\t"
      "addc.cc.u32 %3, %18, %33;\n\t"
      "addc.cc.u32 %4, %19, %34;\n\t"
      "addc.cc.u32 %5, %20, %35;\n\t"
      "addc.cc.u32 %6, %21, %36;\n\t"
      "addc.cc.u32 %7, %22, %37;\n\t"
      "addc.cc.u32 %8, %23, %38;\n\t"
      "addc.cc.u32 %9, %24, %39;\n\t"
      "addc.cc.u32 %10, %25, %40;\n\t"
      "addc.cc.u32 %11, %26, %41;\n\t"
      "addc.cc.u32 %12, %27, %42;\n\t"
      "addc.cc.u32 %13, %28, %43;\n\t"
      "addc.u32 %14, %29, %44;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11]), "=r"(s[12]), "=r"(s[13]), "=r"(s[14])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(a[12]), "r"(a[13]), "r"(a[14]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]), "r"(b[12]), "r"(b[13]), "r"(b[14]));
}
__device__ __forceinline__ void add_run16(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  asm(
      "add.cc.u32 %0, %16, %32;\n\t"
      "addc.cc.u32 %1, %17, %33;\n\t"
      "addc.cc.u32 %2, %18, %34;\n\t"
      "addc.cc.u32 %3, %19, %35;\n\t"
      "addc.cc.u32 %4, %20, %36;\n\t"
      "addc.cc.u32 %5, %21, %37;\n\t"
      "addc.cc.u32 %6, %22, %38;\n\t"
      "addc.cc.u32 %7, %23, %39;\n\t"
      "addc.cc.u32 %8, %24, %40;\n\t"
      "addc.cc.u32 %9, %25, %41;\n\t"
      "addc.cc.u32 %10, %26, %42;\n\t"
      "addc.cc.u32 %11, %27, %43;\n\t"
      "addc.cc.u32 %12, %28, %44;\n\t"
      "addc.cc.u32 %13, %29, %45;\n\t"
      "addc.cc.u32 %14, %30, %46;\n\t"
      "addc.u32 %15, %31, %47;\n\t"
      : "=r"(s[0]), "=r"(s[1]), "=r"(s[2]), "=r"(s[3]), "=r"(s[4]), "=r"(s[5]), "=r"(s[6]), "=r"(s[7]), "=r"(s[8]), "=r"(s[9]), "=r"(s[10]), "=r"(s[11]), "=r"(s[12]), "=r"(s[13]), "=r"(s[14]), "=r"(s[15])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(a[4]), "r"(a[5]), "r"(a[6]), "r"(a[7]), "r"(a[8]), "r"(a[9]), "r"(a[10]), "r"(a[11]), "r"(a[12]), "r"(a[13]), "r"(a[14]), "r"(a[15]), "r"(b[0]), "r"(b[1]), "r"(b[2]), "r"(b[3]), "r"(b[4]), "r"(b[5]), "r"(b[6]), "r"(b[7]), "r"(b[8]), "r"(b[9]), "r"(b[10]), "r"(b[11]), "r"(b[12]), "r"(b[13]), "r"(b[14]), "r"(b[15]));
}
template <int N>
__device__ __forceinline__ void add_run(uint32_t *s, const uint32_t *a, const uint32_t *b) {
  static_assert(N >= 1 && N <= 16, "run length");
#define NGIA_RUN(K) \
  if constexpr (N == K) add_run##K(s, a, b);
  NGIA_RUN(1) NGIA_RUN(2) NGIA_RUN(3) NGIA_RUN(4) NGIA_RUN(5) NGIA_RUN(6) NGIA_RUN(7)
  NGIA_RUN(8) NGIA_RUN(9) NGIA_RUN(10) NGIA_RUN(11) NGIA_RUN(12) NGIA_RUN(13) NGIA_RUN(14)
  NGIA_RUN(15) NGIA_RUN(16)
#undef NGIA_RUN
}


// ---- one LCS column step over a run of words ---------------------------------
// lcs_run<N>(v..., m...): for the N words of a row vector, low word first,
//   t = v & m;  s = v + t + carry;  v = s | (v ^ t)
// with the carry rippling through the flag across the run (lop3 and and.b32
// leave it alone).  Each word is read and written in place, so only the words
// and their masks are live (no separate sum array).  Written out for each N.
__device__ __forceinline__ void lcs_run1(uint32_t &v0, uint32_t m0) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %1;\n\t"
      "add.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "}"
      : "+r"(v0)
      : "r"(m0));
}
__device__ __forceinline__ void lcs_run2(uint32_t &v0, uint32_t &v1, uint32_t m0, uint32_t m1) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %2;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %3;\n\t"
      "addc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1)
      : "r"(m0), "r"(m1));
}
__device__ __forceinline__ void lcs_run3(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t m0, uint32_t m1, uint32_t m2) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %3;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %4;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %5;\n\t"
      "addc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2)
      : "r"(m0), "r"(m1), "r"(m2));
}
__device__ __forceinline__ void lcs_run4(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %4;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %5;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %6;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %7;\n\t"
      "addc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3));
}
__device__ __forceinline__ void lcs_run5(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %5;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %6;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %7;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %8;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %9;\n\t"
      "addc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4));
}
__device__ __forceinline__ void lcs_run6(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %6;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %7;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %8;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %9;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %10;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %11;\n\t"
      "addc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5));
}
__device__ __forceinline__ void lcs_run7(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %7;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %8;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %9;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %10;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %11;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %12;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %13;\n\t"
      "addc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6));
}
__device__ __forceinline__ void lcs_run8(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %8;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %9;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %10;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %11;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %12;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %13;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %14;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %15;\n\t"
      "addc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7));
}
__device__ __forceinline__ void lcs_run9(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t &v8, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7, uint32_t m8) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %9;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %10;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %11;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %12;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %13;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %14;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %15;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %16;\n\t"
      "addc.cc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "and.b32 t, %8, %17;\n\t"
      "addc.u32 s, %8, t;\n\t"
      "lop3.b32 %8, s, %8, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7), "+r"(v8)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7), "r"(m8));
}
__device__ __forceinline__ void lcs_run10(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t &v8, uint32_t &v9, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7, uint32_t m8, uint32_t m9) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %10;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %11;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %12;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %13;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %14;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %15;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %16;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %17;\n\t"
      "addc.cc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "and.b32 t, %8, %18;\n\t"
      "addc.cc.u32 s, %8, t;\n\t"
      "lop3.b32 %8, s, %8, t, 0xF6;\n\t"
      "and.b32 t, %9, %19;\n\t"
      "addc.u32 s, %9, t;\n\t"
      "lop3.b32 %9, s, %9, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7), "+r"(v8), "+r"(v9)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7), "r"(m8), "r"(m9));
}
__device__ __forceinline__ void lcs_run11(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t &v8, uint32_t &v9, uint32_t &v10, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7, uint32_t m8, uint32_t m9, uint32_t m10) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %11;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %12;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %13;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %14;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %15;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %16;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %17;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %18;\n\t"
      "addc.cc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "and.b32 t, %8, %19;\n\t"
      "addc.cc.u32 s, %8, t;\n\t"
      "lop3.b32 %8, s, %8, t, 0xF6;\n\t"
      "and.b32 t, %9, %20;\n\t"
      "addc.cc.u32 s, %9, t;\n\t"
      "lop3.b32 %9, s, %9, t, 0xF6;\n\t"
      "and.b32 t, %10, %21;\n\t"
      "addc.u32 s, %10, t;\n\t"
      "lop3.b32 %10, s, %10, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7), "+r"(v8), "+r"(v9), "+r"(v10)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7), "r"(m8), "r"(m9), "r"(m10));
}
__device__ __forceinline__ void lcs_run12(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t &v8, uint32_t &v9, uint32_t &v10, uint32_t &v11, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7, uint32_t m8, uint32_t m9, uint32_t m10, uint32_t m11) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %12;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %13;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %14;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %15;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %16;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %17;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %18;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %19;\n\t"
      "addc.cc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "and.b32 t, %8, %20;\n\t"
      "addc.cc.u32 s, %8, t;\n\t"
      "lop3.b32 %8, s, %8, t, 0xF6;\n\t"
      "and.b32 t, %9, %21;\n\t"
      "addc.cc.u32 s, %9, t;\n\t"
      "lop3.b32 %9, s, %9, t, 0xF6;\n\t"
      "and.b32 t, %10, %22;\n\t"
      "addc.cc.u32 s, %10, t;\n\t"
      "lop3.b32 %10, s, %10, t, 0xF6;\n\t"
      "and.b32 t, %11, %23;\n\t"
      "addc.u32 s, %11, t;\n\t"
      "lop3.b32 %11, s, %11, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7), "+r"(v8), "+r"(v9), "+r"(v10), "+r"(v11)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7), "r"(m8), "r"(m9), "r"(m10), "r"(m11));
}
__device__ __forceinline__ void lcs_run13(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t &v8, uint32_t &v9, uint32_t &v10, uint32_t &v11, uint32_t &v12, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7, uint32_t m8, uint32_t m9, uint32_t m10, uint32_t m11, uint32_t m12) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %13;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %14;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %15;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %16;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %17;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %18;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %19;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %20;\n\t"
      "addc.cc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "and.b32 t, %8, %21;\n\t"
      "addc.cc.u32 s, %8, t;\n\t"
      "lop3.b32 %8, s, %8, t, 0xF6;\n\t"
      "and.b32 t, %9, %22;\n\t"
      "addc.cc.u32 s, %9, t;\n\t"
      "lop3.b32 %9, s, %9, t, 0xF6;\n\t"
      "and.b32 t, %10, %23;\n\t"
      "addc.cc.u32 s, %10, t;\n\t"
      "lop3.b32 %10, s, %10, t, 0xF6;\n\t"
      "and.b32 t, %11, %24;\n\t"
      "addc.cc.u32 s, %11, t;\n\t"
      "lop3.b32 %11, s, %11, t, 0xF6;\n\t"
      "and.b32 t, %12, %25;\n\t"
      "addc.u32 s, %12, t;\n\t"
      "lop3.b32 %12, s, %12, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7), "+r"(v8), "+r"(v9), "+r"(v10), "+r"(v11), "+r"(v12)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7), "r"(m8), "r"(m9), "r"(m10), "r"(m11), "r"(m12));
}
__device__ __forceinline__ void lcs_run14(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t &v8, uint32_t &v9, uint32_t &v10, uint32_t &v11, uint32_t &v12, uint32_t &v13, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7, uint32_t m8, uint32_t m9, uint32_t m10, uint32_t m11, uint32_t m12, uint32_t m13) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %14;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %15;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %16;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %17;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %18;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %19;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %20;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %21;\n\t"
      "addc.cc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "and.b32 t, %8, %22;\n\t"
      "addc.cc.u32 s, %8, t;\n\t"
      "lop3.b32 %8, s, %8, t, 0xF6;\n\t"
      "and.b32 t, %9, %23;\n\t"
      "addc.cc.u32 s, %9, t;\n\t"
      "lop3.b32 %9, s, %9, t, 0xF6;\n\t"
      "and.b32 t, %10, %24;\n\t"
      "addc.cc.u32 s, %10, t;\n\t"
      "lop3.b32 %10, s, %10, t, 0xF6;\n\t"
      "and.b32 t, %11, %25;\n\t"
      "addc.cc.u32 s, %11, t;\n\t"
      "lop3.b32 %11, s, %11, t, 0xF6;\n\t"
      "and.b32 t, %12, %26;\n\t"
      "addc.cc.u32 s, %12, t;\n\t"
      "lop3.b32 %12, s, %12, t, 0xF6;\n\t"
      "and.b32 t, %13, %27;\n\t"
      "addc.u32 s, %13, t;\n\t"
      "lop3.b32 %13, s, %13, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7), "+r"(v8), "+r"(v9), "+r"(v10), "+r"(v11), "+r"(v12), "+r"(v13)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7), "r"(m8), "r"(m9), "r"(m10), "r"(m11), "r"(m12), "r"(m13));
}
__device__ __forceinline__ void lcs_run15(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t &v8, uint32_t &v9, uint32_t &v10, uint32_t &v11, uint32_t &v12, uint32_t &v13, uint32_t &v14, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7, uint32_t m8, uint32_t m9, uint32_t m10, uint32_t m11, uint32_t m12, uint32_t m13, uint32_t m14) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %15;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %16;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %17;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %18;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %19;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %20;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %21;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %22;\n\t"
      "addc.cc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "and.b32 t, %8, %23;\n\t"
      "addc.cc.u32 s, %8, t;\n\t"
      "lop3.b32 %8, s, %8, t, 0xF6;\n\t"
      "and.b32 t, %9, %24;\n\t"
      "addc.cc.u32 s, %9, t;\n\t"
      "lop3.b32 %9, s, %9, t, 0xF6;\n\t"
      "and.b32 t, %10, %25;\n\t"
      "addc.cc.u32 s, %10, t;\n\t"
      "lop3.b32 %10, s, %10, t, 0xF6;\n\t"
      "and.b32 t, %11, %26;\n\t"
      "addc.cc.u32 s, %11, t;\n\t"
      "lop3.b32 %11, s, %11, t, 0xF6;\n\t"
      "and.b32 t, %12, %27;\n\t"
      "addc.cc.u32 s, %12, t;\n\t"
      "lop3.b32 %12, s, %12, t, 0xF6;\n\t"
      "and.b32 t, %13, %28;\n\t"
      "addc.cc.u32 s, %13, t;\n\t"
      "lop3.b32 %13, s, %13, t, 0xF6;\n\t"
      "and.b32 t, %14, %29;\n\t"
      "addc.u32 s, %14, t;\n\t"
      "lop3.b32 %14, s, %14, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7), "+r"(v8), "+r"(v9), "+r"(v10), "+r"(v11), "+r"(v12), "+r"(v13), "+r"(v14)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7), "r"(m8), "r"(m9), "r"(m10), "r"(m11), "r"(m12), "r"(m13), "r"(m14));
}
__device__ __forceinline__ void lcs_run16(uint32_t &v0, uint32_t &v1, uint32_t &v2, uint32_t &v3, uint32_t &v4, uint32_t &v5, uint32_t &v6, uint32_t &v7, uint32_t &v8, uint32_t &v9, uint32_t &v10, uint32_t &v11, uint32_t &v12, uint32_t &v13, uint32_t &v14, uint32_t &v15, uint32_t m0, uint32_t m1, uint32_t m2, uint32_t m3, uint32_t m4, uint32_t m5, uint32_t m6, uint32_t m7, uint32_t m8, uint32_t m9, uint32_t m10, uint32_t m11, uint32_t m12, uint32_t m13, uint32_t m14, uint32_t m15) {
  asm(
      "{\n\t.reg .u32 t, s;\n\t"
      "and.b32 t, %0, %16;\n\t"
      "add.cc.u32 s, %0, t;\n\t"
      "lop3.b32 %0, s, %0, t, 0xF6;\n\t"
      "and.b32 t, %1, %17;\n\t"
      "addc.cc.u32 s, %1, t;\n\t"
      "lop3.b32 %1, s, %1, t, 0xF6;\n\t"
      "and.b32 t, %2, %18;\n\t"
      "addc.cc.u32 s, %2, t;\n\t"
      "lop3.b32 %2, s, %2, t, 0xF6;\n\t"
      "and.b32 t, %3, %19;\n\t"
      "addc.cc.u32 s, %3, t;\n\t"
      "lop3.b32 %3, s, %3, t, 0xF6;\n\t"
      "and.b32 t, %4, %20;\n\t"
      "addc.cc.u32 s, %4, t;\n\t"
      "lop3.b32 %4, s, %4, t, 0xF6;\n\t"
      "and.b32 t, %5, %21;\n\t"
      "addc.cc.u32 s, %5, t;\n\t"
      "lop3.b32 %5, s, %5, t, 0xF6;\n\t"
      "and.b32 t, %6, %22;\n\t"
      "addc.cc.u32 s, %6, t;\n\t"
      "lop3.b32 %6, s, %6, t, 0xF6;\n\t"
      "and.b32 t, %7, %23;\n\t"
      "addc.cc.u32 s, %7, t;\n\t"
      "lop3.b32 %7, s, %7, t, 0xF6;\n\t"
      "and.b32 t, %8, %24;\n\t"
      "addc.cc.u32 s, %8, t;\n\t"
      "lop3.b32 %8, s, %8, t, 0xF6;\n\t"
      "and.b32 t, %9, %25;\n\t"
      "addc.cc.u32 s, %9, t;\n\t"
      "lop3.b32 %9, s, %9, t, 0xF6;\n\t"
      "and.b32 t, %10, %26;\n\t"
      "addc.cc.u32 s, %10, t;\n\t"
      "lop3.b32 %10, s, %10, t, 0xF6;\n\t"
      "and.b32 t, %11, %27;\n\t"
      "addc.cc.u32 s, %11, t;\n\t"
      "lop3.b32 %11, s, %11, t, 0xF6;\n\t"
      "and.b32 t, %12, %28;\n\t"
      "addc.cc.u32 s, %12, t;\n\t"
      "lop3.b32 %12, s, %12, t, 0xF6;\n\t"
      "and.b32 t, %13, %29;\n\t"
      "addc.cc.u32 s, %13, t;\n\t"
      "lop3.b32 %13, s, %13, t, 0xF6;\n\t"
      "and.b32 t, %14, %30;\n\t"
      "addc.cc.u32 s, %14, t;\n\t"
      "lop3.b32 %14, s, %14, t, 0xF6;\n\t"
      "and.b32 t, %15, %31;\n\t"
      "addc.u32 s, %15, t;\n\t"
      "lop3.b32 %15, s, %15, t, 0xF6;\n\t"
      "}"
      : "+r"(v0), "+r"(v1), "+r"(v2), "+r"(v3), "+r"(v4), "+r"(v5), "+r"(v6), "+r"(v7), "+r"(v8), "+r"(v9), "+r"(v10), "+r"(v11), "+r"(v12), "+r"(v13), "+r"(v14), "+r"(v15)
      : "r"(m0), "r"(m1), "r"(m2), "r"(m3), "r"(m4), "r"(m5), "r"(m6), "r"(m7), "r"(m8), "r"(m9), "r"(m10), "r"(m11), "r"(m12), "r"(m13), "r"(m14), "r"(m15));
}
template <int N, typename... A>
__device__ __forceinline__ void lcs_run(A &&...a) {
  static_assert(N >= 1 && N <= 16 && sizeof...(A) == 2 * N, "run length");
#define NGIA_LCS(K) \
  if constexpr (N == K) lcs_run##K(a...);
  NGIA_LCS(1) NGIA_LCS(2) NGIA_LCS(3) NGIA_LCS(4) NGIA_LCS(5) NGIA_LCS(6) NGIA_LCS(7)
  NGIA_LCS(8) NGIA_LCS(9) NGIA_LCS(10) NGIA_LCS(11) NGIA_LCS(12) NGIA_LCS(13) NGIA_LCS(14)
  NGIA_LCS(15) NGIA_LCS(16)
#undef NGIA_LCS
}

}  // namespace ngia
