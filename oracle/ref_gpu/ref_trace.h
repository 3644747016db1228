/* Record kinds of a reference launch trace -- TEST INFRASTRUCTURE ONLY.
 * Written by oracle/ref_gpu/fake_cuda.cpp, read by oracle/ref_replay.cu.
 * Every record starts with its u32 kind; fields follow in the listed order. */
#ifndef HQ_REF_TRACE_H
#define HQ_REF_TRACE_H
#include <stdint.h>

enum { kRefTraceVersion = 1 };

enum RefTraceRecord {
    REC_END = 0,
    REC_INFO = 1,          /* u32 num_qubits */
    REC_MALLOC = 2,        /* u64 fake address, u64 bytes */
    REC_FREE = 3,          /* u64 fake address */
    REC_MEMSET = 4,        /* u64 dst, u32 value, u64 bytes, u64 stream */
    REC_H2D = 5,           /* u64 dst, u64 stream, u32 async, u64 bytes, bytes */
    REC_D2H = 6,           /* u64 src, u64 bytes */
    REC_D2D = 7,           /* u64 dst, u64 src, u64 stream, u64 bytes */
    REC_SYMBOL_H2D = 8,    /* str name, u64 offset, u64 stream, u64 bytes, bytes */
    REC_LAUNCH = 9,        /* str kernel, u32 grid[3], u32 block[3], u64 shmem, u64 stream,
                              u32 nargs, per argument: u32 bytes, u32 is_pointer, bytes */
    REC_SYNC = 10,         /* u64 stream (all ones: the whole device) */
    REC_REGION_BEGIN = 11, /* cudaProfilerStart: start of the reference's "Time Cost" */
    REC_REGION_END = 12,   /* cudaProfilerStop: its end */
    REC_LAYOUT = 13        /* u32 n, i32 pos[n]: physical position of each logical qubit */
};
/* str = u32 length + bytes (no terminator) */

#endif
