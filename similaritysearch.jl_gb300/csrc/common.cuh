// common.cuh -- shared device helpers of libssgpu: (distance, id) keys and the
// thread-private bounded max-heap that every scan kernel uses as its top-k.
//
// Ordering contract.  SimilaritySearch.jl's KnnSorted keeps results sorted by
// distance and inserts an item AFTER existing equal distances, rejecting an
// item equal to the frontier when full (src/pqueue/knnsorted.jl:68-101,163).
// Because ExhaustiveSearch pushes ids in increasing order
// (src/exact/sequential-exhaustive.jl:73-76), the result is the k smallest
// items under the lexicographic order (distance, id).  Here that order is a
// single 64-bit key: the float distance mapped to an order-preserving uint32
// in the high word and the 0-based id in the low word.  Comparing keys is then
// exactly the reference's order, including its tie rule.
#pragma once
#include <cstdint>
#include <cuda_runtime.h>

namespace ssg {

constexpr uint64_t KEY_EMPTY = ~0ull;

// Order-preserving float -> uint32 (for non-NaN floats).  -0.0 is first
// folded onto +0.0, since the reference compares them as equal.
__host__ __device__ __forceinline__ uint32_t float_to_ordered(float f) {
    f = f + 0.0f;  // -0.0 + 0.0 == +0.0 in round-to-nearest
    uint32_t u;
#ifdef __CUDA_ARCH__
    u = __float_as_uint(f);
#else
    __builtin_memcpy(&u, &f, 4);
#endif
    return (u & 0x80000000u) ? ~u : (u | 0x80000000u);
}

__host__ __device__ __forceinline__ float ordered_to_float(uint32_t u) {
    uint32_t b = (u & 0x80000000u) ? (u & 0x7fffffffu) : ~u;
    float f;
#ifdef __CUDA_ARCH__
    f = __uint_as_float(b);
#else
    __builtin_memcpy(&f, &b, 4);
#endif
    return f;
}

// Three-operand minimum / maximum (one instruction on sm_100+; NaN operands
// are ignored like fminf / fmaxf do).
__device__ __forceinline__ float fmin3(float a, float b, float c) {
    float r;
    asm("min.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
__device__ __forceinline__ float fmax3(float a, float b, float c) {
    float r;
    asm("max.f32 %0, %1, %2, %3;" : "=f"(r) : "f"(a), "f"(b), "f"(c));
    return r;
}
// minimum / maximum of 8 values in 4 instructions
__device__ __forceinline__ float fmin8(const float *v) {
    return fmin3(fmin3(v[0], v[1], v[2]), fmin3(v[3], v[4], v[5]), fminf(v[6], v[7]));
}
__device__ __forceinline__ float fmax8(const float *v) {
    return fmax3(fmax3(v[0], v[1], v[2]), fmax3(v[3], v[4], v[5]), fmaxf(v[6], v[7]));
}

__host__ __device__ __forceinline__ uint64_t make_key(float d, uint32_t id0) {
    return (static_cast<uint64_t>(float_to_ordered(d)) << 32) | id0;
}

__host__ __device__ __forceinline__ float key_dist(uint64_t key) {
    return ordered_to_float(static_cast<uint32_t>(key >> 32));
}

__host__ __device__ __forceinline__ uint32_t key_id0(uint64_t key) {
    return static_cast<uint32_t>(key & 0xffffffffu);
}

// Thread-private max-heap of `kk` keys laid out with stride `st` (so the
// heaps of the threads of a block interleave and a warp touching the same
// slot hits distinct banks).  h[0] is the largest kept key == the frontier.
struct Heap {
    uint64_t *h;
    int kk;
    int st;

    __device__ __forceinline__ void init() {
        for (int i = 0; i < kk; ++i) h[i * st] = KEY_EMPTY;
    }
    __device__ __forceinline__ uint64_t top() const { return h[0]; }

    // Replaces the top with `key` (caller checked key < top) and sifts down.
    __device__ __forceinline__ uint64_t replace_top(uint64_t key) {
        int i = 0;
        while (true) {
            int l = 2 * i + 1;
            if (l >= kk) break;
            int c = l;
            uint64_t hc = h[l * st];
            int r = l + 1;
            if (r < kk) {
                uint64_t hr = h[r * st];
                if (hr > hc) { hc = hr; c = r; }
            }
            if (hc <= key) break;
            h[i * st] = hc;
            i = c;
        }
        h[i * st] = key;
        return h[0];
    }

    // In-place heapsort -> ascending keys in h[0 .. kk-1].
    __device__ void sort_ascending() {
        for (int end = kk - 1; end > 0; --end) {
            uint64_t top = h[0];
            uint64_t last = h[end * st];
            h[end * st] = top;
            // sift `last` down from the root within [0, end)
            int i = 0;
            while (true) {
                int l = 2 * i + 1;
                if (l >= end) break;
                int c = l;
                uint64_t hc = h[l * st];
                int r = l + 1;
                if (r < end) {
                    uint64_t hr = h[r * st];
                    if (hr > hc) { hc = hr; c = r; }
                }
                if (hc <= last) break;
                h[i * st] = hc;
                i = c;
            }
            h[i * st] = last;
        }
    }
};

// A thread-private top-kk heap fed through a small per-thread buffer.
//
// A candidate that beats the thread's (possibly stale) frontier is only
// appended to the buffer; whenever any lane of the warp has `trigger` or more
// buffered, the whole warp drains its buffers into its heaps together.  The
// heap sift-downs of the 32 lanes then run side by side instead of one lane at
// a time, which is what made per-candidate heap insertion slow: lanes of a
// warp find candidates at different moments.  Every lane of the warp must
// call maybe_drain() / drain() (lanes without a query simply offer nothing).
struct BufferedTopK {
    Heap H;
    uint64_t *buf;  // per-thread buffer, `cap` entries with stride H.st
    int c;
    uint64_t top;
    float topd;

    __device__ __forceinline__ void init(uint64_t *heap, uint64_t *buffer, int kk, int st) {
        H.h = heap;
        H.kk = kk;
        H.st = st;
        H.init();
        buf = buffer;
        c = 0;
        top = KEY_EMPTY;
        topd = INFINITY;
    }

    // d passed the caller's prefilter (d <= topd) -- append it.
    __device__ __forceinline__ void append(float d, uint32_t id) {
        buf[c * H.st] = make_key(d, id);
        ++c;
    }

    __device__ __forceinline__ void offer(float d, uint32_t id) {
        if (d <= topd) append(d, id);
    }

    __device__ __forceinline__ void drain() {
        int cmax = __reduce_max_sync(0xffffffffu, c);
        for (int r = 0; r < cmax; ++r) {
            if (r < c) {
                const uint64_t key = buf[r * H.st];
                if (key < top) top = H.replace_top(key);
            }
        }
        c = 0;
        topd = (top == KEY_EMPTY) ? INFINITY : key_dist(top);
    }

    __device__ __forceinline__ void maybe_drain(int trigger) {
        if (__any_sync(0xffffffffu, c >= trigger)) drain();
    }
};

// Drains the c entries buffered at buf (stride st) into the heap h and
// returns the new top.  All 32 lanes of the warp call it together, so the lanes'
// sift-downs run side by side.  Kept out of line so a kernel carries one copy
// of the heap loop however many call sites it has (large unrolled epilogues
// otherwise overflow the instruction cache); every argument is a scalar, so
// the call needs no stack.
// Each slot holds a raw append: the 0-based id in its high word and the bits
// of the column's value in its low word; the value is the distance, or its
// negation when NEG.  The key is made here, once per candidate, instead of
// once per appended column.  With a map, the high word is a position and the
// key takes the id map[position].
template <bool NEG>
static __device__ __noinline__ uint64_t heap_drain_raw(uint64_t *h, const uint64_t *buf, int kk, int st, int c,
                                                       uint64_t top, const uint32_t *map = nullptr) {
    const int cmax = __reduce_max_sync(0xffffffffu, c);
    Heap H{h, kk, st};
    for (int r = 0; r < cmax; ++r) {
        if (r < c) {
            const uint64_t raw = buf[r * st];
            const float v = __uint_as_float(static_cast<uint32_t>(raw));
            const uint32_t pos = static_cast<uint32_t>(raw >> 32);
            const uint64_t key = make_key(NEG ? -v : v, map ? map[pos] : pos);
            if (key < top) top = H.replace_top(key);
        }
    }
    return top;
}

// Bitonic sort of P (a power of two) keys in shared memory by the whole block.
__device__ __forceinline__ void block_bitonic_sort(uint64_t *s, int P) {
    for (int size = 2; size <= P; size <<= 1) {
        for (int stride = size >> 1; stride > 0; stride >>= 1) {
            __syncthreads();
            for (int i = threadIdx.x; i < (P >> 1); i += blockDim.x) {
                int pos = 2 * i - (i & (stride - 1));
                int partner = pos + stride;
                bool asc = (pos & size) == 0;
                uint64_t a = s[pos], b = s[partner];
                if ((a > b) == asc) { s[pos] = b; s[partner] = a; }
            }
        }
    }
    __syncthreads();
}

// The shared per-query bound (see ScanArgs::qbound): lowered to `d` by one
// heap, read back by all.
__device__ __forceinline__ void bound_lower(uint32_t *qb, float d) { atomicMin(qb, float_to_ordered(d)); }
__device__ __forceinline__ float bound_read(const uint32_t *qb) {
    const uint32_t u = __ldcg(qb);
    return u == 0xffffffffu ? INFINITY : ordered_to_float(u);
}

inline int next_pow2(int64_t v) {
    int p = 1;
    while (p < v) p <<= 1;
    return p;
}

}  // namespace ssg
