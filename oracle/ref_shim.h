/*
 * Host shim that lets the CUDA C emitted by the reference translator
 * (xentica/core/base.py:254-283 kernel template, :440-499 builders) compile
 * as plain C++ with g++.  Test infrastructure only: it exists so that the
 * reference's own kernels can be run on the CPU to pin the oracle.
 *
 * Every kernel is a grid-stride loop over cells, so running it with
 * blockDim = 1 and gridDim = T, one OpenMP thread per "block", visits every
 * cell exactly once.  The emit and absorb phases only write cells they own,
 * which makes any thread interleaving give the same result.
 */
#pragma once
#include <cmath>
#include <cstdint>
#include <type_traits>

struct int3 { int x, y, z; };
static inline int3 make_int3(int x, int y, int z) { int3 r; r.x = x; r.y = y; r.z = z; return r; }

struct xk_dim3 { unsigned x, y, z; };
extern thread_local xk_dim3 threadIdx;
extern thread_local xk_dim3 blockIdx;
extern xk_dim3 blockDim;
extern xk_dim3 gridDim;

/* CUDA's integer min/max overloads follow the usual arithmetic conversions. */
template <class A, class B> static inline typename std::common_type<A, B>::type min(A a, B b) { return a < b ? a : b; }
template <class A, class B> static inline typename std::common_type<A, B>::type max(A a, B b) { return a > b ? a : b; }
static inline int __popc(unsigned int v) { return __builtin_popcount(v); }

#define __global__ extern "C"
