// Test infrastructure only (the oracle). Never linked into the product.
//
// A minimal OpenCL-C-to-C++ shim so that the reference's own kernel sources
// (chimeraCL/kernels/*.cl) compile unchanged with g++ and run serially on the
// host: one C++ call per work-item, with get_global_id() returning the
// work-item index held in a thread-local counter.  atom_add is a plain
// read-add-write, which is exact for a serial launch.
//
// Strict IEEE evaluation: the recipe compiles with -ffp-contract=off and no
// fast-math, so results are the reference arithmetic without the
// -cl-fast-relaxed-math licence its GPU build takes
// (chimeraCL/methods/generic_methods_cl.py:15).
#pragma once
#include <cmath>
#include <cstddef>
#include <cstdint>

#define __kernel extern "C"
#define __global
#define __constant
#define __local

typedef unsigned int uint;

struct double2 {
  double s0, s1;
};
static inline double2 operator+(double2 a, double2 b) {
  double2 r;
  r.s0 = a.s0 + b.s0;
  r.s1 = a.s1 + b.s1;
  return r;
}

extern thread_local size_t ccl_ref_gid;
static inline size_t get_global_id(int) { return ccl_ref_gid; }
static inline uint atom_add(uint *p, uint v) {
  uint old = *p;
  *p = old + v;
  return old;
}
