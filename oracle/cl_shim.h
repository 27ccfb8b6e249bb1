/*
 * cl_shim.h -- TEST INFRASTRUCTURE ONLY (oracle). Never linked into the product.
 *
 * Lets gcc compile the reference's OpenCL C sources, as they lie in the reference
 * tree (FeynSimul/GPUsrc/kernel.c after kernel.py's %-substitution, and the vendored
 * examples/pyopencl-ranluxcl.cl), as plain C11 on the host CPU.  The result is the
 * reference's own arithmetic run on the CPU: the pin for the oracle restatement and
 * for the golden fixtures under tests/golden/.
 *
 * Execution model: every OpenCL work-item of one NDRange runs as one POSIX thread.
 * barrier() is a barrier across ALL work-items of the launch.  That is a valid (if
 * stronger) implementation of OpenCL's work-group barrier for kernel.c's
 * parallel-path mode, where every work-item executes the same sequence of barriers
 * (kernel.c:633-636, :726-729, :792).  It also fixes the one scheduling-dependent
 * read of the reference (the xorshift "seedG" row read at kernel.c:568-572, which
 * other work-items overwrite at kernel.c:832-835): all reads happen before the first
 * barrier and all write-backs after the last one, i.e. "snapshot" semantics.
 *
 * Compile with: gcc -std=gnu11 -O2 -fsingle-precision-constant -ffp-contract=off
 * (-fsingle-precision-constant mirrors the reference's -cl-single-precision-constant,
 * kernel.py:376-377; <tgmath.h> gives OpenCL's float overloads of sqrt/log/sin/exp).
 */
#ifndef FS_CL_SHIM_H
#define FS_CL_SHIM_H

#include <limits.h>
#include <math.h>
#include <pthread.h>
#include <stddef.h>
#include <stdint.h>
#include <tgmath.h>

typedef unsigned int uint;
typedef unsigned long ulong; /* 64 bit on LP64 (x86_64 and aarch64) */
typedef struct { uint x, y, z, w; } uint4;
typedef struct { float x, y, z, w; } float4;
typedef struct { double x, y, z, w; } double4;

#define __kernel
#define kernel
#define __global
#define global
#define __private
#define __local
#define __constant const
#define CLK_LOCAL_MEM_FENCE 1
#define CLK_GLOBAL_MEM_FENCE 2

typedef struct {
    size_t gid[3], lid[3], grp[3], gsz[3], lsz[3];
} clsh_item_t;

extern _Thread_local clsh_item_t clsh_item;
extern pthread_barrier_t *clsh_barrier;

static inline size_t get_global_id(uint d) { return d < 3 ? clsh_item.gid[d] : 0; }
static inline size_t get_local_id(uint d) { return d < 3 ? clsh_item.lid[d] : 0; }
static inline size_t get_group_id(uint d) { return d < 3 ? clsh_item.grp[d] : 0; }
static inline size_t get_global_size(uint d) { return d < 3 ? clsh_item.gsz[d] : 1; }
static inline size_t get_local_size(uint d) { return d < 3 ? clsh_item.lsz[d] : 1; }
/* Fiber launches (oracle/ref_timing.py): the work-items of one work-group run as fibers on
 * one OS thread, and barrier() hands over to the group's next fiber through this hook. */
static _Thread_local void (*clsh_barrier_hook)(void);
static inline void barrier(int flags)
{
    (void)flags;
    if (clsh_barrier_hook)
        clsh_barrier_hook();
    else
        pthread_barrier_wait(clsh_barrier);
}
/* OpenCL built-ins that plugin code may call (type-generic through tgmath's sqrt) */
#ifndef rsqrt
#define rsqrt(x) (1 / sqrt(x))
#endif
static inline uint atom_inc(volatile uint *p) { return __atomic_fetch_add(p, 1u, __ATOMIC_RELAXED); }

#endif
