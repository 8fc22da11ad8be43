/*
 * shim.h - the OpenCL C builtins the reference kernels use, for compiling
 * them as C++ on the CPU (test infrastructure: the reference run here as a
 * checker and CPU baseline). Work-items run as fibers; barrier() returns
 * control to the work-group scheduler in harness.cpp.
 */
#pragma once
#include <cmath>
#include <cstdint>

typedef uint64_t ulong;
typedef uint32_t uint;

struct double2 {
    double x, y;
    double2() : x(0), y(0) {}
    double2(double v) : x(v), y(v) {}            // OpenCL scalar broadcast
    double2(double a, double b) : x(a), y(b) {}
    double2 operator-() const { return double2(-x, -y); }
};

static inline uint mul_hi(uint a, uint b) { return (uint)(((uint64_t)a * b) >> 32); }
static inline ulong mul_hi(ulong a, ulong b) { return (ulong)(((unsigned __int128)a * b) >> 64); }
static inline ulong clz(ulong x) { return x ? (ulong)__builtin_clzll(x) : 64; }
using std::trunc;

#define __kernel
#define __global
#define __local
#define CLK_LOCAL_MEM_FENCE 1

// work-item context of the running fiber
struct WorkItem {
    ulong global_id, local_id, group_id, global_size;
};
extern thread_local WorkItem cl_wi;
static inline ulong get_global_id(int) { return cl_wi.global_id; }
static inline ulong get_local_id(int) { return cl_wi.local_id; }
static inline ulong get_group_id(int) { return cl_wi.group_id; }
static inline ulong get_global_size(int) { return cl_wi.global_size; }
void barrier(int);
