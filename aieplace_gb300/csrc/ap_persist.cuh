// Persistent launches of the batched form.
//
// A batch of placement instances runs each stage of a trial step (position
// update, WA gradient, bin scatter, density/overflow, field solve, gather)
// as ONE launch over all instances.  The launch executes the blocks of many
// ordinary launches -- "records", one per instance and stage, record r of
// nblk[r] blocks -- as work items of `chunk` consecutive blocks each (record
// r holds items [start[r], start[r + 1])), and its resident blocks pull
// items off a device queue (an atomic head) until the space is exhausted,
// so instances of uneven size share the GPU without per-instance grids, and
// the graph of a trial step holds nine kernel nodes instead of a dozen per
// instance.  A record's blocks run the same body the
// instance's own launch runs (VBlock{id, n} for blockIdx.x / gridDim.x), so
// each instance's results are the same bit for bit as its own launches'.
//
// Records may depend on one another within a launch (the field solve's four
// contractions of one instance): an item of record r first waits until
// every item of dep[r] has finished.  Items are pulled in order and every
// dependency points at a record earlier in the item space, so an awaited
// item was always taken earlier by a running block and the launch cannot
// deadlock, whether or not all its blocks are resident.  Each wait is
// bounded (wait_ns of device time): when it runs out the item records an
// error in *status, skips its body and still counts as finished, and every
// later wait of the launch gives up at once, so the launch ends within about
// one limit and the host reads the status.
#pragma once

#include "ap_common.cuh"

namespace ap {

constexpr int kPersistMaxRecords = 1024;  // records of one persistent launch (start[] held in shared memory)

struct PersistQueue {
    const int *start;          // [n_rec + 1]: first item of each record, start[n_rec] = total
    const int *nblk;           // [n_rec]: blocks of each record's own launch
    int n_rec;
    int chunk;                 // blocks per item (>= 1)
    unsigned int *head;        // next item to take; zero when the launch starts
    const int *dep;            // [n_rec]: record that must finish first, or -1 (null: no dependencies)
    unsigned int *done;        // [n_rec]: finished items per record (with dep)
    unsigned int *status;      // set to kPersistTimeout when a wait gives up
    unsigned long long wait_ns;
    // counters of the launch before this one on the stream (its head, its
    // done[]), zeroed by this launch's first item: that launch has ended
    unsigned int *reset;
    int n_reset;
    // failure injection: every dependency wait targets one item more than
    // the awaited record has, so no wait is ever satisfied
    int never_arrive;
};

constexpr unsigned int kPersistTimeout = 1u;

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned int ld_acquire(const unsigned int *p) {
    unsigned int v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Runs items until the queue is empty.  `body(args, vb, rec)` runs one block
// of record `rec` with all threads of the block; Args is copied into shared
// memory once per change of record.  Blocks of 32 * k threads.
template <class Args, class Body>
__device__ __forceinline__ void persist_loop(const PersistQueue &q, const Args *__restrict__ recs, Body &&body) {
    static_assert(sizeof(Args) % 4 == 0, "argument block of whole words");
    __shared__ int s_start[kPersistMaxRecords + 1];
    __shared__ int s_nblk[kPersistMaxRecords];
    __shared__ __align__(16) Args s_args;
    __shared__ int s_item, s_skip;
    const int tid = threadIdx.x;
    const int n_rec = q.n_rec;
    for (int t = tid; t <= n_rec; t += blockDim.x) {
        s_start[t] = __ldg(q.start + t);
        if (t < n_rec) s_nblk[t] = __ldg(q.nblk + t);
    }
    if (tid == 0) s_item = (int)atomicAdd(q.head, 1u);
    __syncthreads();
    const int total = s_start[n_rec];
    int cur = -1;
    for (;;) {
        const int it = s_item;
        if (it >= total) return;  // uniform
        // the record holding item `it`: the last r with start[r] <= it
        int lo = 0, hi = n_rec - 1;
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (s_start[mid] <= it) lo = mid;
            else hi = mid - 1;
        }
        const int r = lo;
        if (it == 0)
            for (int t = tid; t < q.n_reset; t += blockDim.x) q.reset[t] = 0u;
        // the next item is fetched now and published after the body: its
        // round trip overlaps the work
        unsigned int next = 0u;
        if (tid == 0) next = atomicAdd(q.head, 1u);
        if (r != cur) {
            __syncthreads();  // every thread is done with the previous record's arguments
            const unsigned int *src = reinterpret_cast<const unsigned int *>(recs + r);
            unsigned int *dst = reinterpret_cast<unsigned int *>(&s_args);
            for (int t = tid; t < (int)(sizeof(Args) / 4); t += blockDim.x) dst[t] = __ldg(src + t);
            cur = r;
        }
        if (tid == 0) {
            int skip = 0;
            const int d = q.dep ? __ldg(q.dep + r) : -1;
            if (d >= 0) {
                // every item of record d (done[] counts items)
                const unsigned int want = (unsigned int)(s_start[d + 1] - s_start[d]) + (q.never_arrive ? 1u : 0u);
                const unsigned long long t0 = global_ns();
                while (ld_acquire(q.done + d) < want) {
                    if (ld_acquire(q.status) != 0u || global_ns() - t0 > q.wait_ns) {
                        atomicOr(q.status, kPersistTimeout);
                        skip = 1;
                        break;
                    }
                    __nanosleep(200);
                }
                __threadfence();
            }
            s_skip = skip;
        }
        __syncthreads();
        if (!s_skip) {
            const int nb = s_nblk[r], b0 = (it - s_start[r]) * q.chunk, b1 = min(b0 + q.chunk, nb);
            for (int vb = b0; vb < b1; ++vb) {
                if (vb > b0) __syncthreads();  // the previous block's shared memory is free
                body(s_args, VBlock{vb, nb}, r);
            }
        }
        __syncthreads();
        if (tid == 0) {
            if (q.dep) {
                __threadfence();
                atomicAdd(q.done + r, 1u);
            }
            s_item = (int)next;
        }
        __syncthreads();
    }
}

}  // namespace ap
