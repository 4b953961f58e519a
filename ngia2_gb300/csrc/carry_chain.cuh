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

}  // namespace ngia
