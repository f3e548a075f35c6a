// ltp_kernels.cu -- sm_103a kernels of the batched transaction-processing hot
// path.  One batch runs as
//
//   mark      read/write-set bitmaps per cell (touched, touched twice,
//             written) built with warp-aggregated atomicOr; records every
//             bitmap word the batch touches
//   ids       contended cell = touched twice and written; a block scan over
//             a tile of touched words numbers its contended cells, and one
//             atomic per tile takes the next free range of dense ids
//   dbase     per contended id: the cell's address, width and value before
//             the batch
//   classify  uncontended ops execute in place (one toucher, or no writer);
//             contended ops are compacted in op order as (id, imm, op)
//             records at dense positions
//   sort      stable LSD radix sort of the contended records by id
//   apply     segmented scan of the RMW immediates per id: every op gets
//             base + (sum of earlier RMWs on its cell in TID order); the last
//             op of each cell writes the final value back
//   insert    committed inserts get their rows (per-table ordered prefix)
//   finish    clears exactly the bitmap words and look-back slots the batch
//             used, so the next batch starts clean
//
// This replaces the reference's nine-stage pipeline (register, prefix,
// bitmap compaction, per-row scatter, per-row merge sort, per-row serial
// commit: cuda/src/gpulauncher.cu:755-1116) while keeping its rule that all
// operations on a row (here: a cell) take effect in ascending TID order.
// The priority rule (R1) replaces sort+apply by min-writer-TID / abort /
// execute kernels.
//
// Tuning knobs per batch-size bucket (picked by the autotuner): threads per
// block and ops per thread of mark and classify, the conflict-word width
// (32 or 64 cells per bitmap word), and mark's hot-word pre-check.  Batches
// carry 64- or 32-bit keys.  Stream-launched batch kernels use programmatic
// dependent launch; one persistent cooperative kernel can run a whole list
// of batches instead.
//
// Every spin-wait (decoupled look-back, grid barrier, the debug stall) is
// bounded by the global timer; on expiry the kernel records LTP_E_TIMEOUT
// and returns.  Debug builds (-DLTP_DEBUG_BOUNDS) check scatter indices.
#include <stdint.h>

#include "ltp_internal.cuh"
#include "ltp_trace.h"

namespace ltp {

#define FULL_MASK 0xFFFFFFFFu

constexpr u64 kSpinLimitNs = 2000000000ull;  // 2 s per wait

// The dynamic shared memory of every kernel: the mark phase's tile hash and
// the insert phase's staging use it in turn.
extern __shared__ __align__(16) u32 ltp_dyn_smem[];

__device__ __forceinline__ u64 gtimer() {
    u64 t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ u64 ld_acquire(const u64 *p) {
    u64 v;
    asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(u64 *p, u64 v) {
    asm volatile("st.release.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ u32 ld_acquire32(const u32 *p) {
    u32 v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_release32(u32 *p, u32 v) {
    asm volatile("st.release.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
// Look-back status words pack the flag and the value into one aligned word,
// so a reader that sees the flag sees the value: relaxed accesses suffice
// (no other data is published through them).
__device__ __forceinline__ u64 ld_status(const u64 *p) {
    u64 v;
    asm volatile("ld.relaxed.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_status(u64 *p, u64 v) {
    asm volatile("st.relaxed.gpu.global.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ u32 ld_status32(const u32 *p) {
    u32 v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}
__device__ __forceinline__ void st_status32(u32 *p, u32 v) {
    asm volatile("st.relaxed.gpu.global.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}
__device__ __forceinline__ u32 lanemask_lt() {
    u32 m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}
__device__ __forceinline__ void set_err(Counters *c, int e) { atomicCAS(&c->err, 0, e); }

// Debug builds (-DLTP_DEBUG_BOUNDS) check the index of every scatter into a
// scratch or table array, and of the conflict words, against the array's
// capacity: a violation records LTP_E_DEVICE_ASSERT and skips the access
// instead of trapping.  Release builds compile the checks away.
#ifdef LTP_DEBUG_BOUNDS
__device__ __forceinline__ bool in_bounds(Counters *ctr, u64 idx, u64 cap) {
    if (idx < cap) return true;
    set_err(ctr, LTP_E_DEVICE_ASSERT);
    return false;
}
#define LTP_IN_BOUNDS(ctr, idx, cap) in_bounds((ctr), (u64)(idx), (u64)(cap))
#else
#define LTP_IN_BOUNDS(ctr, idx, cap) true
#endif
__device__ __forceinline__ u64 mix64(u64 z) {
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

// One view of the device error word for the whole block: every thread takes
// the same early exit, so no barrier or full-warp collective is left short.
__device__ __forceinline__ bool block_err(Counters *ctr) {
    __shared__ int s_err;
    __syncthreads();
    if (threadIdx.x == 0) s_err = *(volatile int *)&ctr->err;
    __syncthreads();
    return s_err != 0;
}

// Claims the next tile for the whole block (tiles are handed out in order,
// which is what makes decoupled look-back safe without co-residency).
__device__ __forceinline__ u32 claim_tile(Counters *ctr, int slot) {
    __shared__ u32 s_tile;
    if (threadIdx.x == 0) s_tile = atomicAdd(&ctr->tile_ctr[slot], 1u);
    __syncthreads();
    u32 t = s_tile;
    __syncthreads();
    return t;
}

// ---- decoupled look-back, scalar sums (flag in bits 62-63) ---------------
constexpr u64 kAgg = 1ull << 62, kInc = 2ull << 62, kValMask = (1ull << 62) - 1;

// Publishes a tile's aggregate (tile 0: its inclusive prefix) early ...
__device__ __forceinline__ void lookback_publish(u64 *status, u32 tile, u64 agg) {
    st_status(&status[tile], (tile == 0 ? kInc : kAgg) | agg);
}
// ... and later walks back for the exclusive prefix, then publishes the
// inclusive one.  Bounded: gives up with LTP_E_TIMEOUT after 2 s.
__device__ __forceinline__ u64 lookback_wait(u64 *status, u32 tile, u64 agg, Counters *ctr) {
    constexpr int WIN = 4;  // predecessors read per round trip
    if (tile == 0) return 0;
    u64 excl = 0;
    long long t = (long long)tile - 1;
    const u64 t0 = gtimer();
    for (;;) {
        u64 st[WIN];
#pragma unroll
        for (int j = 0; j < WIN; j++) st[j] = t - j >= 0 ? ld_status(&status[t - j]) : kInc;
        int j = 0;
        bool done = false;
        for (; j < WIN; j++) {
            const u64 f = st[j] >> 62;
            if (f == 0) break;
            excl += st[j] & kValMask;
            if (f == 2) {
                done = true;
                break;
            }
        }
        if (done) break;
        t -= j;
        if (gtimer() - t0 > kSpinLimitNs) {
            set_err(ctr, LTP_E_TIMEOUT);
            return 0;
        }
    }
    st_status(&status[tile], kInc | (excl + agg));
    return excl;
}

// ---- table addressing ------------------------------------------------------
struct OpRef {
    u64 cell;
    char *ptr;
    bool valid;
    bool wide;
};

__device__ __forceinline__ OpRef decode_op(const TablesDev &T, u64 key, u32 w) {
    OpRef r;
    u32 tb = opw_table(w), col = opw_col(w), kind = opw_kind(w);
    r.valid = tb < T.n && kind <= 1u;
    const TableDev &t = T.t[r.valid ? tb : 0];
    r.valid = r.valid && key < T.rows_now[r.valid ? tb : 0] && col < t.n_cols;  // advanced by finish
    r.wide = r.valid && col_wide(t, col);
    r.cell = r.valid ? t.cell_base + key * t.n_cols + col : ~0ull;
    r.ptr = r.valid ? t.data + col_off(t, col) + key * (r.wide ? 8ull : 4ull) : nullptr;
    return r;
}

// Cell values are handled as 64-bit; int32 cells are sign-extended on load and
// truncated on store, which is exactly 32-bit two's-complement arithmetic.
// ---- L2 eviction-priority hints ---------------------------------------------
// Conflict words (the mark kernel's atomics) and their compact view (read
// by classify) are touched by every batch: keep them in L2.  Uncontended
// table cells are touched once: let them leave L2 first.
__device__ __forceinline__ u64 pol_evict_last() {
    u64 p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ u64 pol_evict_first() {
    u64 p;
    asm volatile("createpolicy.fractional.L2::evict_first.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ uint4 ld_word_relaxed(const void *ptr) {
    uint4 v;
    asm volatile("ld.relaxed.gpu.global.v4.u32 {%0, %1, %2, %3}, [%4];"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(ptr)
                 : "memory");
    return v;
}
// Loads of scratch state with an L2 eviction-priority hint.  Coherent (not
// .nc): the persistent kernel writes this state and reads it again within one
// launch, where only the grid barrier's acquire orders the two, and the
// non-coherent path is defined only for data read-only for a whole kernel.
__device__ __forceinline__ uint4 ld_word_hint(const void *ptr, u64 pol) {
    uint4 v;
    asm volatile("ld.global.L2::cache_hint.v4.u32 {%0, %1, %2, %3}, [%4], %5;"
                 : "=r"(v.x), "=r"(v.y), "=r"(v.z), "=r"(v.w)
                 : "l"(ptr), "l"(pol)
                 : "memory");
    return v;
}
// OR into a conflict word with an L2 eviction-priority hint: with the old
// value (atom) or without (red)
__device__ __forceinline__ u32 atom_or_hint(u32 *p, u32 v, u64 pol) {
    u32 old;
    asm volatile("atom.global.or.L2::cache_hint.b32 %0, [%1], %2, %3;" : "=r"(old) : "l"(p), "r"(v), "l"(pol) : "memory");
    return old;
}
__device__ __forceinline__ u64 atom_or_hint(u64 *p, u64 v, u64 pol) {
    u64 old;
    asm volatile("atom.global.or.L2::cache_hint.b64 %0, [%1], %2, %3;" : "=l"(old) : "l"(p), "l"(v), "l"(pol) : "memory");
    return old;
}
__device__ __forceinline__ void red_or_hint(u32 *p, u32 v, u64 pol) {
    asm volatile("red.global.or.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void red_or_hint(u64 *p, u64 v, u64 pol) {
    asm volatile("red.global.or.L2::cache_hint.b64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st_word_hint(void *ptr, uint4 v, u64 pol) {
    asm volatile("st.global.L2::cache_hint.v4.u32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(ptr), "r"(v.x), "r"(v.y), "r"(v.z),
                 "r"(v.w), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ uint2 ld_view_hint(const void *ptr, u64 pol) {
    uint2 v;
    asm volatile("ld.global.L2::cache_hint.v2.u32 {%0, %1}, [%2], %3;"
                 : "=r"(v.x), "=r"(v.y)
                 : "l"(ptr), "l"(pol)
                 : "memory");
    return v;
}
// ---- programmatic dependent launch -------------------------------------------
// The batch kernels are launched with programmatic stream serialization, so a
// kernel may be launched while its predecessor drains.  Each one first waits
// for the predecessor grid's completion and memory (griddepcontrol.wait; a
// no-op for a launch without the attribute), then lets its own successor be
// launched: the successor's launch and block placement overlap this kernel's
// run, and its blocks wait in turn before their first access.
__device__ __forceinline__ void pdl_begin() {
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

// ---- conflict words ----------------------------------------------------------
// A conflict word covers 32 cells (WordState, 16 B: touched, written and
// touched-twice masks and a spare word) or 64 cells (WordState64, 32 B:
// written and touched-twice masks in its first 16 bytes, then the touched
// mask and a spare).  Both take 16 bytes per 32 cells,
// so one scratch buffer serves either width; the width is a tuning knob of
// the stream and graph launches (the persistent kernel uses 32).
//
// The ids kernel also writes a compact view of every word that holds a
// contended cell: its contended mask (written & touched twice) and its first
// dense id -- 8 B per 32 cells (uint2), 16 B per 64 (uint4) in the cview
// buffer.  Words without a contended cell keep the cleared view {0, 0}.  The
// executing kernels read only the view: half the footprint of the words (42 MB
// for 2^24 x 10 cells) stays in L2 far better while the table streams past.
// The finish kernel clears the views through the contended cells' list.
struct WordState64 {
    u64 wbits, multi, touch;
    u64 pad;
};

template <int WB>
struct Wd;
template <>
struct Wd<32> {
    typedef u32 T;
    static constexpr int kShift = 5;
    struct V {
        u32 wbits, multi, prefix;
    };
    static __device__ __forceinline__ V load(const Scratch &s, u64 w) {  // masks only (prefix 0)
        const uint4 v = *reinterpret_cast<const uint4 *>(&s.words[w]);
        return V{v.y, v.z, 0u};
    }
    // written and touched-twice masks, as the mark kernel's pre-check reads them
    static __device__ __forceinline__ void load_relaxed(const Scratch &s, u64 w, T *wbits, T *multi) {
        const uint4 v = ld_word_relaxed(&s.words[w]);
        *wbits = v.y;
        *multi = v.z;
    }
    static __device__ __forceinline__ T *touch(const Scratch &s, u64 w) { return &s.words[w].touch; }
    static __device__ __forceinline__ T *wbits(const Scratch &s, u64 w) { return &s.words[w].wbits; }
    static __device__ __forceinline__ T *multi(const Scratch &s, u64 w) { return &s.words[w].multi; }
    static __device__ __forceinline__ void clear(const Scratch &s, u64 w) {
        *reinterpret_cast<uint4 *>(&s.words[w]) = make_uint4(0u, 0u, 0u, 0u);
    }
    static __device__ __forceinline__ void clear_hint(const Scratch &s, u64 w, u64 pol) {
        st_word_hint(&s.words[w], make_uint4(0u, 0u, 0u, 0u), pol);
    }
    // the compact view, as V{contended mask, all ones, first id}
    static __device__ __forceinline__ V load_view(const Scratch &s, u64 w, u64 pol) {
        const uint2 v = ld_view_hint(&s.cview[w], pol);
        return V{v.x, ~0u, v.y};
    }
    static __device__ __forceinline__ V load_view_ro(const Scratch &s, u64 w) {
        const uint2 v = s.cview[w];
        return V{v.x, ~0u, v.y};
    }
    static __device__ __forceinline__ void set_view(const Scratch &s, u64 w, T cw, u32 first) {
        s.cview[w] = make_uint2(cw, first);
    }
    static __device__ __forceinline__ void clear_view(const Scratch &s, u64 w) { s.cview[w] = make_uint2(0u, 0u); }
    static __device__ __forceinline__ u64 n_words(const Scratch &s) { return s.n_words; }
    static __device__ __forceinline__ int popc(T x) { return __popc(x); }
    static __device__ __forceinline__ int ffs(T x) { return __ffs(x); }
};
template <>
struct Wd<64> {
    typedef u64 T;
    static constexpr int kShift = 6;
    struct V {
        u64 wbits, multi;
        u32 prefix;
    };
    static __device__ __forceinline__ WordState64 *at(const Scratch &s, u64 w) {
        return reinterpret_cast<WordState64 *>(s.words) + w;
    }
    static __device__ __forceinline__ V load(const Scratch &s, u64 w) {  // masks only (prefix 0)
        const WordState64 *p = at(s, w);
        return V{p->wbits, p->multi, 0u};
    }
    static __device__ __forceinline__ void load_relaxed(const Scratch &s, u64 w, T *wbits, T *multi) {
        const uint4 a = ld_word_relaxed(at(s, w));
        *wbits = ((u64)a.y << 32) | a.x;
        *multi = ((u64)a.w << 32) | a.z;
    }
    static __device__ __forceinline__ T *touch(const Scratch &s, u64 w) { return &at(s, w)->touch; }
    static __device__ __forceinline__ T *wbits(const Scratch &s, u64 w) { return &at(s, w)->wbits; }
    static __device__ __forceinline__ T *multi(const Scratch &s, u64 w) { return &at(s, w)->multi; }
    static __device__ __forceinline__ void clear(const Scratch &s, u64 w) {
        uint4 *p = reinterpret_cast<uint4 *>(at(s, w));
        p[0] = make_uint4(0u, 0u, 0u, 0u);
        p[1] = make_uint4(0u, 0u, 0u, 0u);
    }
    static __device__ __forceinline__ void clear_hint(const Scratch &s, u64 w, u64 pol) {
        uint4 *p = reinterpret_cast<uint4 *>(at(s, w));
        st_word_hint(p, make_uint4(0u, 0u, 0u, 0u), pol);
        st_word_hint(p + 1, make_uint4(0u, 0u, 0u, 0u), pol);
    }
    static __device__ __forceinline__ uint4 *view(const Scratch &s, u64 w) { return reinterpret_cast<uint4 *>(s.cview) + w; }
    static __device__ __forceinline__ V load_view(const Scratch &s, u64 w, u64 pol) {
        const uint4 v = ld_word_hint(view(s, w), pol);
        return V{((u64)v.y << 32) | v.x, ~0ull, v.z};
    }
    static __device__ __forceinline__ V load_view_ro(const Scratch &s, u64 w) {
        const uint4 v = *view(s, w);
        return V{((u64)v.y << 32) | v.x, ~0ull, v.z};
    }
    static __device__ __forceinline__ void set_view(const Scratch &s, u64 w, T cw, u32 first) {
        *view(s, w) = make_uint4((u32)cw, (u32)(cw >> 32), first, 0u);
    }
    static __device__ __forceinline__ void clear_view(const Scratch &s, u64 w) { *view(s, w) = make_uint4(0u, 0u, 0u, 0u); }
    // 64-cell words over the same buffer: half as many, rounded up
    static __device__ __forceinline__ u64 n_words(const Scratch &s) { return (s.n_words + 1) / 2; }
    static __device__ __forceinline__ int popc(T x) { return __popcll(x); }
    static __device__ __forceinline__ int ffs(T x) { return __ffsll((long long)x); }
};

__device__ __forceinline__ long long load_cell_hint(const char *p, bool wide, u64 pol) {
    if (wide) {
        long long v;
        asm volatile("ld.global.L2::cache_hint.b64 %0, [%1], %2;" : "=l"(v) : "l"(p), "l"(pol) : "memory");
        return v;
    }
    int v;
    asm volatile("ld.global.L2::cache_hint.b32 %0, [%1], %2;" : "=r"(v) : "l"(p), "l"(pol) : "memory");
    return (long long)v;
}
__device__ __forceinline__ void store_cell_hint(char *p, bool wide, long long v, u64 pol) {
    if (wide) asm volatile("st.global.L2::cache_hint.b64 [%0], %1, %2;" ::"l"(p), "l"(v), "l"(pol) : "memory");
    else asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(p), "r"((int)v), "l"(pol) : "memory");
}

__device__ __forceinline__ long long load_cell(const char *p, bool wide) {
    return wide ? *reinterpret_cast<const long long *>(p) : (long long)*reinterpret_cast<const int32_t *>(p);
}
__device__ __forceinline__ void store_cell(char *p, bool wide, long long v) {
    if (wide) *reinterpret_cast<long long *>(p) = v;
    else *reinterpret_cast<int32_t *>(p) = (int32_t)v;
}
__device__ __forceinline__ void store_out(const BatchDev &b, u64 i, long long v) {
    b.out[i] = (int32_t)v;
    if (b.out64) b.out64[i] = v;
}

// Output of op i (a valid read or RMW) at full width: ops on int64 cells
// keep it in out64, ops on int32 cells only in out.
__device__ __forceinline__ long long op_value(const BatchDev &b, const TablesDev &T, u64 i) {
    const u32 w = b.opw[i], tb = opw_table(w);
    const bool wide = b.out64 && tb < T.n && col_wide(T.t[tb], opw_col(w));
    return wide ? b.out64[i] : (long long)b.out[i];
}

__device__ __forceinline__ char *cell_ptr(const TablesDev &T, u64 cell, bool *wide) {
    u32 k = 0;
    for (u32 i = 1; i < T.n; i++)
        if (cell >= T.t[i].cell_base) k = i;
    const TableDev &t = T.t[k];
    const u64 local = cell - t.cell_base;
    // 32-bit division whenever the table's cell numbers fit (the usual case)
    const u64 row = local < (1ull << 32) ? (u64)((u32)local / t.n_cols) : local / t.n_cols;
    const u32 col = (u32)(local - row * t.n_cols);
    *wide = col_wide(t, col);
    return t.data + col_off(t, col) + row * (*wide ? 8ull : 4ull);
}

__device__ __forceinline__ u32 op_tid(const BatchDev &b, u64 i);

// An insert's payload row holds one int32 slot per int32 column and two
// (low word first) per int64 column.
__device__ __forceinline__ u64 insert_slots(const TableDev &t) { return (u64)t.n_cols + (u64)__popcll(t.wide); }

// A linked insert (link distance d = low 10 bits of the immediate, d > 0)
// takes column `col` of its new row from the output of op i - d, which must
// be a read or read-modify-write of the same transaction.
__device__ __forceinline__ u32 insert_link(u32 w) { return (u32)opw_imm(w) & 0x3FFu; }
__device__ __forceinline__ bool insert_link_ok(const BatchDev &b, const TableDev &t, u64 i, u32 w) {
    const u32 d = insert_link(w);
    if (!d) return true;
    if (opw_col(w) >= t.n_cols || d > i) return false;
    const u32 tid = op_tid(b, i);
    // fixed-length batches carry ops_per_txn (their txn_first buffer is not loaded)
    const u64 first = b.ops_per_txn ? (u64)tid * b.ops_per_txn : (u64)b.txn_first[tid];
    return i - d >= first && opw_kind(b.opw[i - d]) <= LTP_OP_ADD;
}

// Is the cell contended (touched twice and written)?  If so, *m is its dense id.
template <int WB>
__device__ __forceinline__ bool contended_id(const Scratch &s, u64 cell, u32 *m) {
    typedef typename Wd<WB>::T WT;
    const typename Wd<WB>::V v = Wd<WB>::load_view_ro(s, cell >> Wd<WB>::kShift);
    const WT cw = v.wbits & v.multi, bit = (WT)1 << (cell & (WB - 1));
    *m = v.prefix + Wd<WB>::popc(cw & (bit - 1));
    return (cw & bit) != 0;
}

// Key of op i (the batch carries 64-bit or 32-bit keys; the choice is
// uniform over the batch).
__device__ __forceinline__ u64 op_key(const BatchDev &b, u64 i) { return b.keys32 ? (u64)b.keys32[i] : b.keys[i]; }
__device__ __forceinline__ u64 op_key_stream(const BatchDev &b, u64 i) {  // read once: evict first
    return b.keys32 ? (u64)__ldcs(&b.keys32[i]) : __ldcs(&b.keys[i]);
}

__device__ __forceinline__ u32 op_tid(const BatchDev &b, u64 i) {
    return b.ops_per_txn ? (u32)(i / b.ops_per_txn) : b.op_txn[i];
}

// ============================================================================
// mark: read/write-set bitmaps
//
// Each tile of BLOCK*IPT ops is staged in a shared-memory hash keyed by
// bitmap word: every op ORs its cell bit into the word's "touched" mask and,
// when the bit was already there, into its "touched twice" mask; RMW ops also
// set the "written" mask.  The tile then issues one global atomicOr per
// distinct word and flag -- under Zipf skew a hot word costs one atomic per
// tile instead of one per op, which removes the same-address serialisation
// at L2 that otherwise dominates the batch.
// ============================================================================
constexpr u32 kEmptyKey = 0xFFFFFFFFu;

__device__ __forceinline__ u32 hash_word(u32 w) { return (w * 0x9E3779B1u) ^ (w >> 15); }

// dynamic shared memory of the mark hash: key + touched, touched-twice and
// written masks per slot, 2 slots per op of the tile
template <int BLOCK, int IPT, int WB>
constexpr size_t mark_smem_bytes() { return 2ull * BLOCK * IPT * (4 + 3 * (WB / 8)); }

// A batch whose keys and opwords take most of the L2 cannot keep them there
// until classify reads them again: mark streams them (evict-first), so they
// do not push the conflict words out (Zipf, 2^24 ops with 32-bit keys, 134
// MB: mark 0.300 -> 0.285 ms).  A smaller batch loads them normally and
// classify finds them in L2 (order entry, 5.5 M ops with 64-bit keys, 66 MB:
// streaming them cost 2%).
constexpr u64 kStreamOpsBytes = 96ull << 20;

template <int BLOCK, int IPT, int WB>
__device__ __forceinline__ void phase_mark(const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr) {
    typedef typename Wd<WB>::T WT;
    // A batch with at least twice as many ops as conflict words touches
    // most of them: ids and finish will visit every word in address order,
    // so no touched-word list is built, only its length counted, per warp
    // across its tiles (the list cost a global atomic round trip and two
    // barriers per tile: Zipf mark 0.278 -> 0.272 ms).  Every block records
    // the choice before it touches a word, so finish clears every word
    // whenever any block marked one.
    const bool no_list = b.n_ops >= 2ull * Wd<WB>::n_words(s);
    if (no_list && threadIdx.x == 0) ctr->dense = 1u;
    if (block_err(ctr)) return;
    const bool precheck = (b.flags & LTP_TUNE_MARK_PRECHECK) != 0u;
    // the words stay in L2 from batch to batch (hot words are touched by
    // every batch); the executing kernels read only the compact view
    const u64 pol_keep = pol_evict_last();
    const bool stream_ops = b.n_ops * ((b.keys32 ? 4ull : 8ull) + 4ull) > kStreamOpsBytes;
    constexpr u32 TILE = (u32)BLOCK * IPT;
    static_assert(kInsTile % TILE == 0, "a mark tile lies inside one insert tile");
    constexpr u32 H = 2 * TILE;  // at most TILE distinct words: load factor <= 1/2
    u32 *hk = ltp_dyn_smem;  // H keys, then 3 * H masks (dynamic)
    WT *ht = reinterpret_cast<WT *>(hk + H), *hd = ht + H, *hw = hd + H;
    __shared__ u32 s_ins[LTP_MAX_TABLES];  // insert ops of the tile per table
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u64 n = b.n_ops;
    u64 n_first = 0;  // no_list: first-touched words of this warp's share of the tiles
    // range of the words each warp flushed, kept in shared memory across tiles
    __shared__ u32 s_wlo[BLOCK / 32], s_whi1[BLOCK / 32];
    __shared__ u32 s_wide;  // some op of the block is on an int64 cell
    if (lane == 0) {
        s_wlo[warp] = 0xFFFFFFFFu;
        s_whi1[warp] = 0u;
    }
    if (threadIdx.x == 0) s_wide = 0u;
    for (u64 base = (u64)blockIdx.x * TILE; base < n; base += (u64)gridDim.x * TILE) {
        for (u32 i = threadIdx.x; i < H; i += BLOCK) {
            hk[i] = kEmptyKey;
            ht[i] = 0u;
            hd[i] = 0u;
            hw[i] = 0u;
        }
        if (threadIdx.x < LTP_MAX_TABLES) s_ins[threadIdx.x] = 0u;
        const u64 wbase = base + (u64)warp * 32 * IPT;
        u64 key[IPT];
        u32 w[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            u64 i = wbase + (u64)k * 32 + lane;
            key[k] = i < n ? (stream_ops ? op_key_stream(b, i) : op_key(b, i)) : 0;
            w[k] = i < n ? (stream_ops ? __ldcs(&b.opw[i]) : b.opw[i]) : 0xFFFFFFFFu;
        }
        __syncthreads();
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const u64 i = wbase + (u64)k * 32 + lane;
            if (i >= n) continue;
            if (opw_kind(w[k]) == LTP_OP_INSERT) {  // appends a row: no existing cell to mark
                const u32 tb = opw_table(w[k]);
                if (tb < T.n && key[k] + insert_slots(T.t[tb]) <= b.payload_len && insert_link_ok(b, T.t[tb], i, w[k])) {
                    atomicAdd(&s_ins[tb], 1u);
                } else {
                    atomicMax(&ctr->bad_op, ~i);
                    set_err(ctr, LTP_E_BADARG);
                }
                continue;
            }
            OpRef r = decode_op(T, key[k], w[k]);
            if (!r.valid) {  // record the lowest malformed op (stored inverted)
                atomicMax(&ctr->bad_op, ~i);
                set_err(ctr, LTP_E_BADARG);
                continue;
            }
            if (r.wide) s_wide = 1u;
            const u32 word = (u32)(r.cell >> Wd<WB>::kShift);
            const WT bit = (WT)1 << (r.cell & (WB - 1));
            u32 slot = hash_word(word) & (H - 1);
            for (u32 probe = 0; probe < H; probe++) {
                u32 cur = hk[slot];
                if (cur == kEmptyKey) cur = atomicCAS(&hk[slot], kEmptyKey, word);
                if (cur == kEmptyKey || cur == word) break;
                slot = (slot + 1) & (H - 1);
            }
            if (atomicOr(&ht[slot], bit) & bit) atomicOr(&hd[slot], bit);
            if (opw_kind(w[k]) != LTP_OP_READ) atomicOr(&hw[slot], bit);
        }
        __syncthreads();
        if (threadIdx.x < LTP_MAX_TABLES && s_ins[threadIdx.x]) {
            // per table: the batch's inserts, and those of this tile's insert tile
            atomicAdd(&ctr->ins_total[threadIdx.x], s_ins[threadIdx.x]);
            const u64 slot = (base / kInsTile) * LTP_MAX_TABLES + threadIdx.x;
            if (LTP_IN_BOUNDS(ctr, slot, s.cap_tiles * LTP_MAX_TABLES)) atomicAdd(&s.ins_pre[slot], s_ins[threadIdx.x]);
        }
        // flush: every thread issues the touch atomics of all its slots before
        // consuming any result, so the returning atomics overlap
        constexpr int SPT = H / BLOCK;
        u32 fw[SPT];
        WT ft[SPT], old[SPT];
#pragma unroll
        for (int q = 0; q < SPT; q++) {
            const u32 j = threadIdx.x + q * BLOCK;
            fw[q] = hk[j];
            ft[q] = ht[j];
        }
        // a word whose touched, touched-twice and written bits already hold
        // what this tile adds needs no atomic (hot words, after their first
        // tiles); the bits only ever grow, so a stale read merely costs an
        // atomic that was not needed.  Only words this tile touched more than
        // once are checked first: a word touched once per tile is usually
        // cold, and the read would only add a round trip before its atomic.
        WT cur_w[SPT], cur_m[SPT];  // the word's written and touched-twice bits as read
#pragma unroll
        for (int q = 0; q < SPT; q++) {
            const u32 j = threadIdx.x + q * BLOCK;
            const bool hot = precheck && fw[q] != kEmptyKey && (hd[j] != 0 || (ft[q] & (ft[q] - 1)) != 0);
            cur_w[q] = cur_m[q] = 0;
            if (hot) Wd<WB>::load_relaxed(s, fw[q], &cur_w[q], &cur_m[q]);
        }
        {
            u32 lo = 0xFFFFFFFFu, hi1 = 0u;
#pragma unroll
            for (int q = 0; q < SPT; q++)
                if (fw[q] != kEmptyKey) {
                    lo = min(lo, fw[q]);
                    hi1 = max(hi1, fw[q] + 1u);
                }
            lo = __reduce_min_sync(FULL_MASK, lo);
            hi1 = __reduce_max_sync(FULL_MASK, hi1);
            if (lane == 0) {
                s_wlo[warp] = min(s_wlo[warp], lo);
                s_whi1[warp] = max(s_whi1[warp], hi1);
            }
        }
        u32 dmask = 0;  // slots that issued their atomics
#pragma unroll
        for (int q = 0; q < SPT; q++) {
            const u32 j = threadIdx.x + q * BLOCK;
            const bool need = fw[q] != kEmptyKey && ((ft[q] & ~cur_m[q]) || (hw[j] & ~cur_w[q])) &&
                              LTP_IN_BOUNDS(ctr, fw[q], Wd<WB>::n_words(s));
            old[q] = need ? atom_or_hint(Wd<WB>::touch(s, fw[q]), ft[q], pol_keep) : 0;
            if (need) dmask |= 1u << q;
        }
        u32 fmask = 0, nfirst = 0;
#pragma unroll
        for (int q = 0; q < SPT; q++) {
            const u32 j = threadIdx.x + q * BLOCK;
            if (dmask & (1u << q)) {
                const WT m = (old[q] & ft[q]) | hd[j];
                if (m & ~cur_m[q]) red_or_hint(Wd<WB>::multi(s, fw[q]), m, pol_keep);
                if (hw[j] & ~cur_w[q]) red_or_hint(Wd<WB>::wbits(s, fw[q]), hw[j], pol_keep);
                if (old[q] == 0) {
                    fmask |= 1u << q;
                    nfirst++;
                }
            }
        }
        if (no_list) {  // count the first-touched words only, per warp across its tiles
            n_first += __reduce_add_sync(FULL_MASK, nfirst);
            __syncthreads();
            continue;
        }
        // first-touched words go to the touched-word list with one global
        // atomic per tile (a per-warp counter on one address serialises)
        u32 incl = nfirst;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const u32 v = __shfl_up_sync(FULL_MASK, incl, d);
            if (lane >= d) incl += v;
        }
        __shared__ u32 s_wtot[BLOCK / 32];
        __shared__ u64 s_base;
        if (lane == 31) s_wtot[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            u32 run = 0;
            for (int i = 0; i < BLOCK / 32; i++) {
                const u32 c = s_wtot[i];
                s_wtot[i] = run;
                run += c;
            }
            s_base = run ? atomicAdd(&ctr->n_tw, (u64)run) : 0ull;
        }
        __syncthreads();
        u64 pos = s_base + s_wtot[warp] + (incl - nfirst);
#pragma unroll
        for (int q = 0; q < SPT; q++)
            if (fmask & (1u << q)) {
                if (LTP_IN_BOUNDS(ctr, pos, s.cap_ops)) s.tw_list[pos] = fw[q];
                pos++;
            }
        __syncthreads();
    }
    if (no_list && lane == 0 && n_first) atomicAdd(&ctr->n_tw, n_first);  // one add per warp
    // the range of touched words, one pair of atomics per block: ids and
    // finish stream over it in address order when it is densely touched
    // (a batch on one table of a context with larger ones touches a small
    // part of the word space)
    __syncthreads();
    if (threadIdx.x == 0) {
        u32 wlo = s_wlo[0], whi1 = s_whi1[0];
        for (int i = 1; i < BLOCK / 32; i++) {
            wlo = min(wlo, s_wlo[i]);
            whi1 = max(whi1, s_whi1[i]);
        }
        if (whi1) {
            atomicMax(&ctr->wlo_inv, ~wlo);
            atomicMax(&ctr->whi1, whi1);
        }
        if (s_wide) atomicOr(&ctr->wide_ops, 1u);
    }
}

template <int BLOCK, int IPT, int WB>
__global__ void __launch_bounds__(BLOCK) k_mark(BatchDev b, TablesDev T, Scratch s, Counters *ctr) {
    pdl_begin();
    phase_mark<BLOCK, IPT, WB>(b, T, s, ctr);
}

// ============================================================================
// ids: dense ids of contended cells (touched twice and written)
// ============================================================================
// When a batch touches more than a quarter of the conflict words between
// the lowest and the highest it touched, the ids scan and the clean-up
// stream over that range in address order instead of visiting the
// touched-word list in first-touch (random) order.  A batch with at least
// twice as many ops as words is taken as such without counting: mark builds
// no list for it (see phase_mark).
__device__ __forceinline__ u64 touched_lo(const Counters *ctr) { return ctr->whi1 ? (u64)~ctr->wlo_inv : 0ull; }
__device__ __forceinline__ u64 touched_hi(const Counters *ctr) { return (u64)ctr->whi1; }
__device__ __forceinline__ bool ids_dense(const Counters *ctr) {
    return ctr->dense || ctr->n_tw * 4 > touched_hi(ctr) - touched_lo(ctr);
}

// Per contended cell: its address width (bit 63 of dcell marks an int64
// cell), its value before the batch, and (priority rule) the min-writer slot.
__device__ __forceinline__ void phase_dbase(const TablesDev &T, const Scratch &s, Counters *ctr, bool priority) {
    if (block_err(ctr)) return;
    const u64 M = ctr->M;
    for (u64 m = (u64)blockIdx.x * blockDim.x + threadIdx.x; m < M; m += (u64)gridDim.x * blockDim.x) {
        if (!LTP_IN_BOUNDS(ctr, m, s.cap_ops)) continue;
        const u64 cell = s.dcell[m];
        bool wide_c;
        const char *cp = cell_ptr(T, cell, &wide_c);
        if (wide_c) s.dcell[m] = cell | (1ull << 63);
        s.dbase[m] = load_cell(cp, wide_c);
        if (priority) s.dminw[m] = 0xFFFFFFFFu;
    }
}

__global__ void __launch_bounds__(256) k_dbase(TablesDev T, Scratch s, Counters *ctr, int priority) {
    pdl_begin();
    phase_dbase(T, s, ctr, priority != 0);
}

template <int BLK, int WB>
__device__ __forceinline__ void phase_ids(const TablesDev &T, const Scratch &s, Counters *ctr) {
    typedef typename Wd<WB>::T WT;
    constexpr u32 IPT = kIdsTile / BLK;
    if (block_err(ctr)) return;
    const bool dense = ids_dense(ctr);
    const u64 wlo = touched_lo(ctr), whi = min(touched_hi(ctr), Wd<WB>::n_words(s));
    const u64 n = dense ? (whi > wlo ? whi - wlo : 0ull) : ctr->n_tw;
    const u32 tiles = (u32)((n + kIdsTile - 1) / kIdsTile);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ u32 s_warp[BLK / 32];
    __shared__ u64 s_prefix;
    if (blockIdx.x == 0 && threadIdx.x < T.n) {  // room for this batch's inserts?
        const u32 tb = threadIdx.x;
        if (T.rows_now[tb] + ctr->ins_total[tb] > T.t[tb].row_limit) set_err(ctr, LTP_E_CAPACITY);
    }
    for (u32 tile = blockIdx.x; tile < tiles; tile += gridDim.x) {  // tiles wait for no other tile
        u32 wd[IPT];
        WT cw[IPT];
        u32 cnt = 0;
        // striped arrangement (coalesced loads); a thread's entries get
        // consecutive ids -- any bijection onto 0..M-1 serves as ids
        const u64 t0 = (u64)tile * kIdsTile + threadIdx.x;
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            u64 j = t0 + (u64)k * BLK;
            wd[k] = j < n ? (dense ? (u32)(wlo + j) : s.tw_list[j]) : 0u;
            if (j < n) {
                const typename Wd<WB>::V v = Wd<WB>::load(s, wd[k]);
                cw[k] = v.wbits & v.multi;
            } else {
                cw[k] = 0;
            }
            cnt += Wd<WB>::popc(cw[k]);
        }
        // block exclusive scan of cnt
        u32 incl = cnt;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            u32 v = __shfl_up_sync(FULL_MASK, incl, d);
            if (lane >= d) incl += v;
        }
        if (lane == 31) s_warp[warp] = incl;
        __syncthreads();
        if (threadIdx.x == 0) {
            u32 run = 0;
            for (int i = 0; i < BLK / 32; i++) {
                u32 c = s_warp[i];
                s_warp[i] = run;
                run += c;
            }
            // ids need only be a bijection onto 0..M-1 with each word's ids
            // consecutive: a tile takes the next free range with one atomic
            // and waits for no other tile (M ends as the total)
            s_prefix = run ? atomicAdd(&ctr->M, run) : 0u;
        }
        __syncthreads();
        u64 pre = s_prefix + s_warp[warp] + (incl - cnt);
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            u64 j = t0 + (u64)k * BLK;
            if (j < n && cw[k]) {
                Wd<WB>::set_view(s, wd[k], cw[k], (u32)pre);
                WT bits = cw[k];
                while (bits) {  // the cells' values are read by k_dbase, fully parallel
                    const int bpos = Wd<WB>::ffs(bits) - 1;
                    bits &= bits - 1;
                    if (LTP_IN_BOUNDS(ctr, pre, s.cap_ops)) s.dcell[pre] = ((u64)wd[k] << Wd<WB>::kShift) | (u64)bpos;
                    pre++;
                }
            }
        }
        __syncthreads();
    }
}

template <int WB>
__global__ void __launch_bounds__(kIdsBlock) k_ids(TablesDev T, Scratch s, Counters *ctr) {
    pdl_begin();
    phase_ids<kIdsBlock, WB>(T, s, ctr);
}

// ============================================================================
// classify (ordered rule): execute uncontended ops, compact contended ones,
// and histogram the contended ids' radix digits for the sort
// ============================================================================
// Radix passes over the contended ids: 8 bits each, at least one pass as soon
// as there is a contended cell.
// Contended-op records.  Packed (fewer than 2^20 contended cells and at most
// 2^24 ops): id << 44 | imm20 << 24 | op -- the RMW immediate travels with
// the record (a read carries 0, which is what it adds).  Otherwise:
// id << 32 | rmw << 31 | op, and the immediate is read from the opword.
__device__ __forceinline__ bool rec_packed(u32 M, u64 n_ops) { return M < (1u << 20) && n_ops <= (1ull << 24); }
__device__ __forceinline__ int rec_shift(bool packed) { return packed ? 44 : 32; }
__device__ __forceinline__ u32 rec_id(u64 e, bool packed) { return (u32)(e >> rec_shift(packed)); }
__device__ __forceinline__ u32 rec_op(u64 e, bool packed) {
    return packed ? (u32)e & 0xFFFFFFu : (u32)e & 0x7FFFFFFFu;
}

__device__ __forceinline__ int sort_passes_dev(u32 M) {
    if (M == 0) return 0;
    const int bits = M == 1 ? 1 : 32 - __clz(M - 1);
    return (bits + 7) / 8;
}

template <int BLOCK, int IPT, int WB>
__device__ __forceinline__ void phase_classify(const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr) {
    typedef typename Wd<WB>::T WT;
    if (block_err(ctr)) return;
    constexpr int NW = BLOCK / 32;
    constexpr u64 TILE = (u64)BLOCK * IPT;
    const u64 n = b.n_ops;
    const u32 tiles = (u32)((n + TILE - 1) / TILE);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int passes = sort_passes_dev(ctr->M);
    const bool packed = rec_packed(ctr->M, n);
    const u64 pol_keep = pol_evict_last(), pol_once = pol_evict_first();
    __shared__ u32 s_wcnt[NW];
    __shared__ u32 s_run;
    __shared__ u64 s_pbase;
    __shared__ u32 s_hist[kMaxPasses][256];
    for (int i = threadIdx.x; i < kMaxPasses * 256; i += BLOCK) (&s_hist[0][0])[i] = 0;
    __syncthreads();
    for (;;) {
        const u32 tile = claim_tile(ctr, SLOT_CLASSIFY);
        if (tile >= tiles) break;
        const u64 wbase = (u64)tile * TILE + (u64)warp * 32 * IPT;
        u64 key[IPT];
        u32 w[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            u64 i = wbase + (u64)k * 32 + lane;
            key[k] = i < n ? op_key_stream(b, i) : 0;
            w[k] = i < n ? __ldcs(&b.opw[i]) : 0xFFFFFFFFu;
        }
        OpRef r[IPT];
        typename Wd<WB>::V ws[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            u64 i = wbase + (u64)k * 32 + lane;
            r[k] = decode_op(T, key[k], w[k]);
            r[k].valid = r[k].valid && i < n;
            if (r[k].valid) ws[k] = Wd<WB>::load_view(s, r[k].cell >> Wd<WB>::kShift, pol_keep);
            else ws[k].wbits = ws[k].multi = 0, ws[k].prefix = 0;
        }
        u64 rec[IPT];
        u32 wcnt = 0, lpos[IPT];
        bool con[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            const WT bit = (WT)1 << (r[k].cell & (WB - 1));
            const WT cw = ws[k].wbits & ws[k].multi;
            const u64 i = wbase + (u64)k * 32 + lane;
            con[k] = r[k].valid && (cw & bit);
            const u32 m = ws[k].prefix + Wd<WB>::popc(cw & (bit - 1));
            rec[k] = packed ? ((u64)m << 44) |
                                  ((u64)(opw_kind(w[k]) == LTP_OP_ADD ? ((u32)opw_imm(w[k]) & 0xFFFFFu) : 0u) << 24) |
                                  (u64)(u32)i
                            : ((u64)m << 32) | ((u64)(opw_kind(w[k]) == LTP_OP_ADD) << 31) | (u64)(u32)i;
            const u32 bal = __ballot_sync(FULL_MASK, con[k]);
            lpos[k] = wcnt + __popc(bal & lanemask_lt());
            wcnt += __popc(bal);
            if (con[k])  // digit histograms for the radix sort
                for (int p = 0; p < passes; p++) atomicAdd(&s_hist[p][(m >> (8 * p)) & 255u], 1u);
        }
        if (lane == 0) s_wcnt[warp] = wcnt;
        __syncthreads();
        if (threadIdx.x == 0) {
            // the tile's contended records go to the dense list in op order:
            // its count is published now, its offset is looked back for after
            // the uncontended ops have executed
            u32 run = 0;
            for (int i = 0; i < NW; i++) {
                u32 c = s_wcnt[i];
                s_wcnt[i] = run;
                run += c;
            }
            s_run = run;
            lookback_publish(s.st_cls, tile, run);
            if (run) atomicAdd(&ctr->n_c, (u64)run);
        }
        // uncontended ops execute in place; an uncontended read's cell is never
        // written in this batch, an uncontended RMW is its cell's only op
        // (the cell is read only once the word says the op runs here: reading
        // it speculatively for contended ops costs more than the overlap saves)
        long long val[IPT];
#pragma unroll
        for (int k = 0; k < IPT; k++)
            if (r[k].valid && !con[k])
                val[k] = load_cell_hint(r[k].ptr, r[k].wide, pol_once);
#pragma unroll
        for (int k = 0; k < IPT; k++) {
            if (r[k].valid && !con[k]) {
                long long v = val[k];
                if (opw_kind(w[k]) == LTP_OP_ADD) {
                    v = (long long)((u64)v + (u64)(long long)opw_imm(w[k]));
                    if (!r[k].wide) v = (int32_t)v;  // int32 cells wrap at 32 bits
                    store_cell_hint(r[k].ptr, r[k].wide, v, pol_once);
                }
                const u64 i = wbase + (u64)k * 32 + lane;
                __stcs(&b.out[i], (int32_t)v);
                if (b.out64 && r[k].wide) b.out64[i] = v;  // int32 cells: widened from out on fetch
            }
        }
        if (threadIdx.x == 0) s_pbase = lookback_wait(s.st_cls, tile, s_run, ctr);
        __syncthreads();
        const u64 pbase = s_pbase + s_wcnt[warp];
#pragma unroll
        for (int k = 0; k < IPT; k++)
            if (con[k] && LTP_IN_BOUNDS(ctr, pbase + lpos[k], s.cap_ops)) s.list[0][pbase + lpos[k]] = rec[k];
        __syncthreads();
    }
    for (int i = threadIdx.x; i < passes * 256; i += BLOCK) {
        const u32 c = (&s_hist[0][0])[i];
        if (c) atomicAdd(&(&ctr->hist[0][0])[i], c);
    }
}

template <int BLOCK, int IPT, int WB>
// register budget per thread: 40 up to 2 ops per thread, 48 up to 4, 96
// above, so that 64-bit cell values do not cut the resident blocks
__global__ void __launch_bounds__(BLOCK, 65536 / (BLOCK * (IPT <= 2 ? 40 : IPT <= 4 ? 48 : 96))) k_classify(BatchDev b, TablesDev T,
                                                                                          Scratch s, Counters *ctr) {
    pdl_begin();
    phase_classify<BLOCK, IPT, WB>(b, T, s, ctr);
}

// ============================================================================
// sort: stable LSD radix sort of the contended records by id (8-bit digits);
// each tile ranks its records per digit, finds its digit offsets by
// decoupled look-back, stages the records in shared memory in digit order
// and writes every digit's run with coalesced stores
// ============================================================================
// Stable LSD radix pass (8-bit digit P) over the dense contended records.
// Per tile of kSortTile records: warp ranking by peer masks (8 ballots or
// one match.any give the lanes that share a digit; the group's lowest lane adds the group size to
// the warp's shared counter, whose old value is the group's offset -- a
// warp's shared-memory atomics take effect in program order, which keeps
// the ranks stable), per-digit decoupled look-back over a window of eight
// predecessor tiles with relaxed loads, shared-memory staging so every
// digit's run leaves as coalesced stores.
template <int BLK>
__device__ __forceinline__ void phase_sort_pass(const int P, const Scratch &s, Counters *ctr, u64 n_ops) {
    static_assert(BLK == 256, "one thread per radix digit");
    constexpr u32 SIPT = kSortTile / BLK;
    constexpr int WIN = 8;
    if (block_err(ctr)) return;
    const int passes = sort_passes_dev(ctr->M);
    if (P >= passes) return;
    const u64 n = ctr->n_c;
    const u32 tiles = (u32)((n + kSortTile - 1) / kSortTile);
    const u64 *src = s.list[P & 1];
    u64 *dst = s.list[(P + 1) & 1];
    u32 *status = s.st_sort[P & 1];
    if (P >= 1) {  // the previous pass is complete: recycle its look-back slots
        u32 *other = s.st_sort[(P + 1) & 1];
        for (u64 j = (u64)blockIdx.x * BLK + threadIdx.x; j < (u64)tiles * 256; j += (u64)gridDim.x * BLK)
            other[j] = 0;
    }
    constexpr int NW = BLK / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const u32 tid = threadIdx.x;
    __shared__ u32 s_start[256];
    __shared__ u32 s_cnt[NW][256];  // per-warp digit counts, then per-warp offsets
    __shared__ u32 s_base[256];     // global position of the tile's first record of each digit
    __shared__ u32 s_loc[256];      // tile-local position of each digit's first record
    __shared__ u32 s_wsum[NW];
    __shared__ u64 s_stage[kSortTile];
    {  // global start of every digit: exclusive scan of the histogram
        const u32 h = ctr->hist[P][tid];
        u32 incl = h;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const u32 v = __shfl_up_sync(FULL_MASK, incl, d);
            if (lane >= d) incl += v;
        }
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        u32 off = 0;
        for (int i = 0; i < warp; i++) off += s_wsum[i];
        s_start[tid] = off + incl - h;
        __syncthreads();
    }
    const int shift = rec_shift(rec_packed(ctr->M, n_ops)) + 8 * P;
    for (;;) {
        const u32 tile = claim_tile(ctr, SLOT_SORT0 + P);
        if (tile >= tiles) break;
        for (u32 i = tid; i < NW * 256; i += BLK) (&s_cnt[0][0])[i] = 0;
        const u32 tcnt = (u32)min((u64)kSortTile, n - (u64)tile * kSortTile);
        const u32 lbase = (u32)warp * 32 * SIPT;
        u64 e[SIPT];
#pragma unroll
        for (int k = 0; k < SIPT; k++) {
            const u32 li = lbase + (u32)k * 32 + lane;
            e[k] = li < tcnt ? __ldcs(&src[(u64)tile * kSortTile + li]) : ~0ull;
        }
        __syncthreads();
        u32 rank[SIPT], old[SIPT], lead[SIPT];
#pragma unroll
        for (int k = 0; k < SIPT; k++) {
            const bool v = lbase + (u32)k * 32 + lane < tcnt;
            const u32 d = (u32)(e[k] >> shift) & 255u;
            // lanes holding the same digit (an empty lane matches only
            // itself): eight ballots on the first pass, whose records are
            // still in op order; match.any on the later ones (measured
            // faster there, slower on the first)
            u32 peers;
            if (P == 0) {
                peers = __ballot_sync(FULL_MASK, v);
#pragma unroll
                for (int bit = 0; bit < 8; bit++) {
                    const u32 m = __ballot_sync(FULL_MASK, (d >> bit) & 1u);
                    peers &= ((d >> bit) & 1u) ? m : ~m;
                }
            } else {
                peers = __match_any_sync(FULL_MASK, v ? d : 256u + (u32)lane);
            }
            const u32 ld = (u32)__ffs(peers) - 1u;
            u32 o = 0;
            if (v && (u32)lane == ld) o = atomicAdd(&s_cnt[warp][d], (u32)__popc(peers));
            old[k] = o;
            lead[k] = ld & 31u;
            rank[k] = __popc(peers & lanemask_lt());
        }
#pragma unroll
        for (int k = 0; k < SIPT; k++) rank[k] += __shfl_sync(FULL_MASK, old[k], lead[k]);
        __syncthreads();
        // thread tid owns digit tid: per-warp offsets, the tile's count, and
        // its aggregate published before the local scan
        u32 run = 0;
#pragma unroll
        for (int w = 0; w < NW; w++) {
            const u32 c = s_cnt[w][tid];
            s_cnt[w][tid] = run;
            run += c;
        }
        u32 *slot = &status[(u64)tile * 256 + tid];
        st_status32(slot, (tile == 0 ? (2u << 30) : (1u << 30)) | run);
        {  // tile-local digit starts: exclusive scan of the tile's digit counts
            u32 incl = run;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const u32 v = __shfl_up_sync(FULL_MASK, incl, d);
                if (lane >= d) incl += v;
            }
            if (lane == 31) s_wsum[warp] = incl;
            __syncthreads();
            u32 off = 0;
            for (int i = 0; i < warp; i++) off += s_wsum[i];
            s_loc[tid] = off + incl - run;
        }
        // per-digit look-back over windows of WIN predecessors
        u32 excl = 0;
        if (tile > 0) {
            long long t = (long long)tile - 1;
            const u64 t0 = gtimer();
            bool done = false;
            while (!done && t >= 0) {
                u32 st[WIN];
#pragma unroll
                for (int j = 0; j < WIN; j++)
                    st[j] = t - j >= 0 ? ld_status32(&status[(u64)(t - j) * 256 + tid]) : (2u << 30);
                int j = 0;
                for (; j < WIN; j++) {
                    const u32 f = st[j] >> 30;
                    if (f == 0) break;
                    excl += st[j] & 0x3FFFFFFFu;
                    if (f == 2) {
                        done = true;
                        break;
                    }
                }
                if (done) break;
                t -= j;
                if (gtimer() - t0 > kSpinLimitNs) {
                    set_err(ctr, LTP_E_TIMEOUT);
                    break;
                }
            }
            st_status32(slot, (2u << 30) | (excl + run));
        }
        s_base[tid] = s_start[tid] + excl;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < SIPT; k++) {
            if (lbase + (u32)k * 32 + lane < tcnt) {
                const u32 d = (u32)(e[k] >> shift) & 255u;
                s_stage[s_loc[d] + s_cnt[warp][d] + rank[k]] = e[k];
            }
        }
        __syncthreads();
        for (u32 p = tid; p < tcnt; p += BLK) {
            const u64 x = s_stage[p];
            const u32 d = (u32)(x >> shift) & 255u;
            if (LTP_IN_BOUNDS(ctr, s_base[d] + (p - s_loc[d]), s.cap_ops)) dst[s_base[d] + (p - s_loc[d])] = x;
        }
        __syncthreads();
    }
}

template <int P>
__global__ void __launch_bounds__(kSortBlock, 3) k_sort_pass(Scratch s, Counters *ctr, u64 n_ops) {
    pdl_begin();
    phase_sort_pass<kSortBlock>(P, s, ctr, n_ops);
}

// ============================================================================
// apply: segmented scan of RMW immediates per contended cell, write-back
// ============================================================================
// look-back status: bits 62-63 flag, bit 61 "tile holds a segment head",
// bits 0-60 sum since the last head.  S is the scan type: u32 when every
// column is int32 (wrapping int32 arithmetic), u64 when some column is int64;
// a 64-bit sum of signed 20-bit immediates over < 2^32 ops stays below 2^52
// in magnitude, so 61 sign-extended bits hold it exactly.
constexpr u64 kSum61 = (1ull << 61) - 1ull;
template <typename S>
__device__ __forceinline__ S unpack_sum(u64 x) {
    return (S)(u64)(((long long)(x << 3)) >> 3);
}

template <int BLK, typename S>
__device__ __forceinline__ void phase_apply(const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr) {
    constexpr u32 AIPT = kApplyTile / BLK;
    constexpr bool WIDE = sizeof(S) == 8;
    if (block_err(ctr)) return;
    const u64 n = ctr->n_c;
    const u32 tiles = (u32)((n + kApplyTile - 1) / kApplyTile);
    // a select, not s.list[runtime index]: indexing the parameter's pointer
    // pair at run time copies the whole Scratch to every thread's stack
    const u64 *list = (sort_passes_dev(ctr->M) & 1) ? s.list[1] : s.list[0];
    const bool packed = rec_packed(ctr->M, b.n_ops);
    constexpr int NW = BLK / 32;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ u32 s_wf[NW];
    __shared__ S s_ws[NW];
    __shared__ u32 s_tf;
    __shared__ S s_ts;
    for (;;) {
        const u32 tile = claim_tile(ctr, SLOT_APPLY);
        if (tile >= tiles) break;
        const u64 wbase = (u64)tile * kApplyTile + (u64)warp * 32 * AIPT;
        u64 e[AIPT];
        S sv[AIPT];
        bool sf[AIPT];
        bool tail[AIPT];
#pragma unroll
        for (int k = 0; k < AIPT; k++) {
            u64 i = wbase + (u64)k * 32 + lane;
            e[k] = i < n ? __ldcs(&list[i]) : ~0ull;
        }
        u32 cf = 0;
        S cs = 0;  // running carry within the warp
        // the warp's neighbours outside its own 32 x AIPT run
        const u64 before_w = (lane == 0 && wbase > 0 && wbase - 1 < n) ? list[wbase - 1] : ~0ull;
        const u64 wend = wbase + 32ull * AIPT;
        const u64 after_w = (lane == 31 && wend < n) ? list[wend] : ~0ull;
#pragma unroll
        for (int k = 0; k < AIPT; k++) {
            const u64 i = wbase + (u64)k * 32 + lane;
            const bool v = i < n;
            const u32 m = rec_id(e[k], packed);
            // element i - 1 is lane - 1 of this row, or lane 31 of the previous row
            u64 prev = __shfl_up_sync(FULL_MASK, e[k], 1);
            const u64 prev_row = __shfl_sync(FULL_MASK, k > 0 ? e[k > 0 ? k - 1 : 0] : before_w, k > 0 ? 31 : 0);
            if (lane == 0) prev = prev_row;
            u64 next = __shfl_down_sync(FULL_MASK, e[k], 1);
            const u64 next_row = __shfl_sync(FULL_MASK, k + 1 < (int)AIPT ? e[k + 1 < (int)AIPT ? k + 1 : k] : after_w,
                                             k + 1 < (int)AIPT ? 0 : 31);
            if (lane == 31) next = next_row;
            const bool head = v && (i == 0 || rec_id(prev, packed) != m);
            tail[k] = v && (i + 1 == n || rec_id(next, packed) != m);
            S val = 0;
            if (v) {
                if (packed) val = (S)(long long)(((int)((u32)(e[k] >> 24) << 12)) >> 12);  // sign-extend 20 bits
                else if ((e[k] >> 31) & 1ull) val = (S)(long long)opw_imm(__ldg(&b.opw[(u32)e[k] & 0x7FFFFFFFu]));
            }
            u32 f = head ? 1u : 0u;
            S sum = val;
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                S us = __shfl_up_sync(FULL_MASK, sum, d);
                u32 uf = __shfl_up_sync(FULL_MASK, f, d);
                if (lane >= d) {
                    if (!f) sum += us;
                    f |= uf;
                }
            }
            if (!f) sum += cs;
            f |= cf;
            sv[k] = sum;
            sf[k] = f != 0;
            cs = __shfl_sync(FULL_MASK, sum, 31);
            cf = __shfl_sync(FULL_MASK, f, 31);
        }
        if (lane == 0) {
            s_wf[warp] = cf;
            s_ws[warp] = cs;
        }
        __syncthreads();
        if (warp == 0) {
            // lane 0: exclusive prefix over warps and the tile's aggregate;
            // then the whole warp looks back, 32 predecessors per round trip
            u32 af = 0;
            S as = 0;
            if (lane == 0) {
                for (int w = 0; w < NW; w++) {
                    u32 f = s_wf[w];
                    S sm = s_ws[w];
                    s_wf[w] = af;
                    s_ws[w] = as;
                    if (f) {
                        af = 1;
                        as = sm;
                    } else {
                        as += sm;
                    }
                }
                const u64 agg = ((u64)af << 61) | ((u64)as & kSum61);
                st_status(&s.st_apply[tile], (tile == 0 ? kInc : kAgg) | agg);
            }
            af = __shfl_sync(FULL_MASK, af, 0);
            as = __shfl_sync(FULL_MASK, as, 0);
            u64 *st = s.st_apply;
            u32 ef = 0;
            S es = 0;
            if (tile > 0) {
                long long t = (long long)tile - 1;  // lane j reads predecessor t - j
                const u64 t0 = gtimer();
                for (;;) {
                    const long long q = t - lane;
                    const u64 x = q >= 0 ? ld_status(&st[q]) : kInc;
                    const u32 fl = (u32)(x >> 62);
                    const u32 hb = (u32)((x >> 61) & 1ull);
                    const u32 nr = __ballot_sync(FULL_MASK, fl == 0);               // not yet published
                    const u32 sp = __ballot_sync(FULL_MASK, fl == 2 || (fl != 0 && hb));  // ends the walk
                    const int first_nr = nr ? __ffs(nr) - 1 : 32;
                    const int first_sp = sp ? __ffs(sp) - 1 : 32;
                    const bool stop = first_sp < first_nr;
                    const int upto = stop ? first_sp + 1 : first_nr;  // lanes [0, upto) are summed
                    S v = lane < upto ? unpack_sum<S>(x) : (S)0;
#pragma unroll
                    for (int d = 16; d >= 1; d >>= 1) v += __shfl_xor_sync(FULL_MASK, v, d);
                    es += v;
                    if (stop) {
                        ef = __shfl_sync(FULL_MASK, hb, first_sp);
                        break;
                    }
                    t -= first_nr;
                    if (__shfl_sync(FULL_MASK, (u32)(gtimer() - t0 > kSpinLimitNs), 0)) {
                        if (lane == 0) set_err(ctr, LTP_E_TIMEOUT);
                        break;
                    }
                }
                if (lane == 0) {
                    const u32 incf = af ? 1u : ef;
                    const S incs = af ? as : es + as;
                    st_status(&st[tile], kInc | ((u64)incf << 61) | ((u64)incs & kSum61));
                }
            }
            if (lane == 0) {
                s_tf = ef;
                s_ts = es;
            }
        }
        __syncthreads();
        // carry into this warp = combine(tile exclusive, warp exclusive)
        const u32 wf = s_wf[warp];
        const S ws = s_ws[warp];
        const S carry = wf ? ws : s_ts + ws;
#pragma unroll
        for (int k = 0; k < AIPT; k++) {
            const u64 i = wbase + (u64)k * 32 + lane;
            if (i < n) {
                const u32 m = rec_id(e[k], packed);
                const S tot = sf[k] ? sv[k] : sv[k] + carry;
                const u32 op = rec_op(e[k], packed);
                if (!LTP_IN_BOUNDS(ctr, op, b.n_ops) || !LTP_IN_BOUNDS(ctr, m, s.cap_ops)) continue;
                if (!WIDE) {  // every cell is int32: out64 (if any) is widened from out on fetch
                    const int32_t val = (int32_t)((u32)s.dbase[m] + (u32)tot);
                    b.out[op] = val;
                    if (tail[k]) {
                        bool wd;
                        char *p = cell_ptr(T, s.dcell[m], &wd);
                        *reinterpret_cast<int32_t *>(p) = val;
                    }
                } else {
                    // bit 63 of dcell marks an int64 cell
                    const u64 dc = s.dcell[m];
                    long long val = (long long)((u64)s.dbase[m] + (u64)tot);
                    if (!(dc >> 63)) val = (int32_t)val;
                    b.out[op] = (int32_t)val;
                    if ((dc >> 63) && b.out64) b.out64[op] = val;  // int32 cells: widened from out on fetch
                    if (tail[k]) {
                        bool wd;
                        char *p = cell_ptr(T, dc & ~(1ull << 63), &wd);
                        store_cell(p, wd, val);
                    }
                }
            }
        }
        __syncthreads();
    }
}

template <typename S>
__global__ void __launch_bounds__(kApplyBlock, 4) k_apply(BatchDev b, TablesDev T, Scratch s, Counters *ctr) {
    pdl_begin();
    phase_apply<kApplyBlock, S>(b, T, s, ctr);
}

// In a context with int64 columns the scan is 64-bit only for a batch that
// has an op on an int64 cell (mark records it); a batch on int32 tables
// alone scans in 32 bits, as in a context without int64 columns.
__global__ void __launch_bounds__(kApplyBlock, 4) k_apply_auto(BatchDev b, TablesDev T, Scratch s, Counters *ctr) {
    pdl_begin();
    if (*(volatile u32 *)&ctr->wide_ops) phase_apply<kApplyBlock, u64>(b, T, s, ctr);
    else phase_apply<kApplyBlock, u32>(b, T, s, ctr);
}

// ============================================================================
// priority rule (R1): min writer TID per contended cell, aborts, execute
// ============================================================================
template <int WB>
__device__ __forceinline__ void phase_r1_minw(const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr) {
    if (block_err(ctr)) return;
    const u64 n = b.n_ops;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i - threadIdx.x < n; i += (u64)gridDim.x * blockDim.x) {
        bool act = false, con = false;
        u32 m = 0, tid = 0;
        if (i < n) {
            const u32 w = b.opw[i];
            OpRef r = decode_op(T, op_key(b, i), w);
            con = r.valid && contended_id<WB>(s, r.cell, &m);
            if (con && opw_kind(w) == LTP_OP_ADD) {
                act = true;
                tid = op_tid(b, i);
            }
        }
        const u32 nc = __popc(__ballot_sync(FULL_MASK, con));
        if ((threadIdx.x & 31) == 0 && nc) atomicAdd(&ctr->n_c, (u64)nc);
        const u32 peers = __match_any_sync(FULL_MASK, act ? m : 0xFFFFFFFFu);
        const u32 mn = __reduce_min_sync(peers, act ? tid : 0xFFFFFFFFu);
        if (act && (threadIdx.x & 31) == (u32)(__ffs(peers) - 1) && LTP_IN_BOUNDS(ctr, m, s.cap_ops))
            atomicMin(&s.dminw[m], mn);
    }
}

template <int WB>
__global__ void __launch_bounds__(256) k_r1_minw(BatchDev b, TablesDev T, Scratch s, Counters *ctr) {
    pdl_begin();
    phase_r1_minw<WB>(b, T, s, ctr);
}

template <int WB>
__device__ __forceinline__ void phase_r1_abort(const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr) {
    if (block_err(ctr)) return;
    const u64 n = b.n_ops;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u32 w = b.opw[i];
        OpRef r = decode_op(T, op_key(b, i), w);
        u32 m;
        if (r.valid && contended_id<WB>(s, r.cell, &m)) {
            const u32 tid = op_tid(b, i);
            if (s.dminw[m] < tid) b.commit[tid] = 0;
        }
    }
}

template <int WB>
__global__ void __launch_bounds__(256) k_r1_abort(BatchDev b, TablesDev T, Scratch s, Counters *ctr) {
    pdl_begin();
    phase_r1_abort<WB>(b, T, s, ctr);
}

template <int WB>
__device__ __forceinline__ void phase_r1_exec(const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr) {
    if (block_err(ctr)) return;
    const u64 n = b.n_ops;
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (u64)gridDim.x * blockDim.x) {
        const u32 w = b.opw[i];
        OpRef r = decode_op(T, op_key(b, i), w);
        if (!r.valid) continue;
        const u32 tid = op_tid(b, i);
        if (!b.commit[tid]) {
            store_out(b, i, 0);
            continue;
        }
        u32 m;
        const bool add = opw_kind(w) == LTP_OP_ADD;
        long long v;
        bool store = add;
        if (contended_id<WB>(s, r.cell, &m)) {
            // A committed op on a contended cell sees the pre-batch value,
            // plus -- when its transaction is the cell's only committed
            // writer (the smallest writing TID) -- the RMWs its own
            // transaction made to the cell before it; only the
            // transaction's last RMW on the cell stores.
            v = s.dbase[m];
            if (s.dminw[m] == tid) {
                const u64 key = op_key(b, i);
                const u32 same = w & 0xFFCu;  // column and table fields
                // fixed-length batches carry ops_per_txn (their txn_first buffer is not loaded)
                const u64 first = b.ops_per_txn ? (u64)tid * b.ops_per_txn : (u64)b.txn_first[tid];
                const u64 end = b.ops_per_txn ? first + b.ops_per_txn : (u64)b.txn_first[tid + 1];
                for (u64 j = first; j < end; j++) {
                    if (j == i) continue;
                    const u32 wj = b.opw[j];
                    if (opw_kind(wj) != LTP_OP_ADD || (wj & 0xFFCu) != same || op_key(b, j) != key) continue;
                    if (j < i) v = (long long)((u64)v + (u64)(long long)opw_imm(wj));
                    else store = false;
                }
            }
        } else {
            v = load_cell(r.ptr, r.wide);
        }
        if (add) v = (long long)((u64)v + (u64)(long long)opw_imm(w));
        if (!r.wide) v = (int32_t)v;
        if (store) store_cell(r.ptr, r.wide, v);
        store_out(b, i, v);
    }
}

template <int WB>
__global__ void __launch_bounds__(256) k_r1_exec(BatchDev b, TablesDev T, Scratch s, Counters *ctr) {
    pdl_begin();
    phase_r1_exec<WB>(b, T, s, ctr);
}

// ============================================================================
// insert: slots for committed inserts, per table, in (TID, op) order -- a
// 16-way ordered prefix sum (warp match_any ranks, per-table decoupled
// look-back) -- then the payload row is copied into its slot
// ============================================================================
// The separate insert kernel copies rows through per-(table, column)
// descriptors kept in its dynamic shared memory after the staging arrays;
// the persistent kernel, whose shared memory every phase shares, keeps the
// flattened per-cell loop (16 KB more there would leave two blocks per SM
// almost no L1).
constexpr u32 kInsPairs = LTP_MAX_TABLES * LTP_MAX_COLS;
constexpr u32 kInsSmemDesc = kInsSmem + kInsPairs * 8 + (kInsPairs + 1) * 4 + kInsPairs * 4;
static_assert(kInsSmem % 8 == 0, "the descriptors' addresses start 8-byte aligned");

template <int BLK, bool DESC>
__device__ __forceinline__ void phase_insert(const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr,
                                             bool prefixed) {
    constexpr u32 IIPT = kInsTile / BLK;
    if (block_err(ctr)) return;
    u32 any = 0;
    for (u32 k = 0; k < T.n; k++) any |= ctr->ins_total[k];
    if (!any) return;
    constexpr int NW = BLK / 32;
    const u64 n = b.n_ops;
    const u32 tiles = (u32)((n + kInsTile - 1) / kInsTile);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ u32 s_wcnt[NW][LTP_MAX_TABLES];
    __shared__ u64 s_base[LTP_MAX_TABLES];
    __shared__ u32 s_tcnt[LTP_MAX_TABLES], s_toff[LTP_MAX_TABLES];
    __shared__ u32 s_item0[LTP_MAX_TABLES + 1];  // first (table, column, row) item of each table
    __shared__ u32 s_pair0[LTP_MAX_TABLES + 1];  // first (table, column) pair of each table
    // staging of the tile's inserts in the dynamic shared memory (kInsSmem bytes)
    u32 *s_off = ltp_dyn_smem;                                                  // [kInsTile] payload offsets
    long long *s_lv = reinterpret_cast<long long *>(ltp_dyn_smem + kInsTile);  // [kInsTile] link values
    unsigned char *s_lc = reinterpret_cast<unsigned char *>(s_lv + kInsTile);  // [kInsTile] link columns
    // DESC: per (table, column) pair of the tile's new rows, its first item,
    // the address of its first new row, and slot | column << 8 | wide << 14
    // | table << 16 -- so that a cell's copy needs no division and no lookup
    // of the table's descriptor (dynamic, after the staging arrays)
    char **s_pdst = reinterpret_cast<char **>(reinterpret_cast<unsigned char *>(ltp_dyn_smem) + kInsSmem);  // [kInsPairs]
    u32 *s_pitem = reinterpret_cast<u32 *>(s_pdst + kInsPairs);  // [kInsPairs + 1]
    u32 *s_pmeta = s_pitem + kInsPairs + 1;                       // [kInsPairs]
    for (;;) {
        const u32 tile = claim_tile(ctr, SLOT_INSERT);
        if (tile >= tiles) break;
        for (u32 i = threadIdx.x; i < NW * LTP_MAX_TABLES; i += BLK) (&s_wcnt[0][0])[i] = 0;
        __syncthreads();
        const u64 wbase = (u64)tile * kInsTile + (u64)warp * 32 * IIPT;
        u32 tb[IIPT], lrank[IIPT];
#pragma unroll
        for (int k = 0; k < IIPT; k++) {
            const u64 i = wbase + (u64)k * 32 + lane;
            bool ins = false;
            u32 t = LTP_MAX_TABLES;
            if (i < n) {
                const u32 w = b.opw[i];
                if (opw_kind(w) == LTP_OP_INSERT) {
                    t = opw_table(w);
                    ins = prefixed || b.commit[op_tid(b, i)] != 0;  // prefixed: every transaction commits
                    if (!ins) store_out(b, i, 0);
                }
            }
            tb[k] = ins ? t : LTP_MAX_TABLES;
            const u32 peers = __match_any_sync(FULL_MASK, tb[k]);
            const u32 before = ins ? s_wcnt[warp][t] : 0u;
            __syncwarp();
            if (ins && lane == __ffs(peers) - 1) s_wcnt[warp][t] = before + __popc(peers);
            __syncwarp();
            lrank[k] = before + __popc(peers & lanemask_lt());
        }
        __syncthreads();
        if (threadIdx.x < LTP_MAX_TABLES) {  // thread t owns table t
            const u32 t = threadIdx.x;
            u32 run = 0;
            for (int w = 0; w < NW; w++) {
                const u32 c = s_wcnt[w][t];
                s_wcnt[w][t] = run;
                run += c;
            }
            u32 *st = s.st_ins;
            u32 excl = 0;
            u32 *slot = &st[(u64)tile * LTP_MAX_TABLES + t];
            if (prefixed) {
                // every transaction commits (ordered rule): the tile's offset
                // is the prefix of the insert counts mark took, no look-back
                excl = s.ins_pre[(u64)tile * LTP_MAX_TABLES + t];
            } else if (tile == 0) {
                st_status32(slot, (2u << 30) | run);
            } else {
                st_status32(slot, (1u << 30) | run);
                long long q = (long long)tile - 1;
                const u64 t0 = gtimer();
                while (q >= 0) {
                    const u32 v = ld_status32(&st[(u64)q * LTP_MAX_TABLES + t]);
                    const u32 f = v >> 30;
                    if (f == 0) {
                        if (gtimer() - t0 > kSpinLimitNs) {
                            set_err(ctr, LTP_E_TIMEOUT);
                            break;
                        }
                        continue;
                    }
                    excl += v & 0x3FFFFFFFu;
                    if (f == 2) break;
                    q--;
                }
                st_status32(slot, (2u << 30) | (excl + run));
            }
            s_base[t] = (t < T.n ? T.rows_now[t] : 0ull) + excl;
            s_tcnt[t] = run;
            if (run) atomicAdd(&ctr->ins_committed[t], run);
        }
        __syncthreads();
        if (threadIdx.x == 0) {  // the tile's inserts, grouped by table, in rank order
            u32 run = 0, items = 0, pairs = 0;
            for (int t = 0; t < LTP_MAX_TABLES; t++) {
                s_toff[t] = run;
                run += s_tcnt[t];
                s_item0[t] = items;
                s_pair0[t] = pairs;
                if ((u32)t < T.n && s_tcnt[t]) {
                    items += s_tcnt[t] * T.t[t].n_cols;
                    pairs += T.t[t].n_cols;
                }
            }
            s_item0[LTP_MAX_TABLES] = items;
            s_pair0[LTP_MAX_TABLES] = pairs;
        }
        __syncthreads();
        if constexpr (DESC) {
            for (u32 q = threadIdx.x; q < s_pair0[LTP_MAX_TABLES]; q += BLK) {  // thread q describes pair q
                u32 t = 0;
                while (s_pair0[t + 1] <= q) t++;
                const TableDev &tab = T.t[t];
                const u32 c = q - s_pair0[t];
                const bool wc = col_wide(tab, c);
                const u32 slot = c + (u32)__popcll(c ? (tab.wide & ((1ull << c) - 1ull)) : 0ull);  // payload slot of column c
                s_pitem[q] = s_item0[t] + c * s_tcnt[t];
                s_pdst[q] = tab.data + col_off(tab, c) + s_base[t] * (wc ? 8ull : 4ull);
                s_pmeta[q] = slot | (c << 8) | ((wc ? 1u : 0u) << 14) | (t << 16);
            }
            if (threadIdx.x == 0) s_pitem[s_pair0[LTP_MAX_TABLES]] = s_item0[LTP_MAX_TABLES];
            __syncthreads();
        }
        // every insert notes its payload row and link; its output is its row id
#pragma unroll
        for (int k = 0; k < IIPT; k++) {
            if (tb[k] < LTP_MAX_TABLES) {
                const u64 i = wbase + (u64)k * 32 + lane;
                const u32 r = s_wcnt[warp][tb[k]] + lrank[k];
                const u32 e = s_toff[tb[k]] + r;
                const u32 w = b.opw[i];
                const u32 d = insert_link(w);
                s_off[e] = (u32)op_key(b, i);
                s_lc[e] = d ? (unsigned char)opw_col(w) : (unsigned char)0xFF;
                s_lv[e] = d ? op_value(b, T, i - d) : 0ll;
                store_out(b, i, (long long)(s_base[tb[k]] + r));
            }
        }
        __syncthreads();
        // every (table, column, row) cell of the tile's new rows is one item,
        // column-major within a table: consecutive threads store consecutive
        // rows of a column, and a thread's items issue their loads together
        const u32 n_items = s_item0[LTP_MAX_TABLES];
        constexpr int U = 4;  // items per thread in flight: their loads issue before their stores
        u32 pr = 0;           // items of a thread only move forward through the pairs (tables)
        for (u32 it0 = threadIdx.x; it0 < n_items; it0 += U * BLK) {
            long long v[U];
            char *dst[U];
            bool wc[U];
#pragma unroll
            for (int q = 0; q < U; q++) {
                const u32 it = it0 + q * BLK;
                dst[q] = nullptr;
                if (it >= n_items) continue;
                u32 t, c, j, slot;
                if constexpr (DESC) {
                    while (s_pitem[pr + 1] <= it) pr++;
                    const u32 meta = s_pmeta[pr];
                    j = it - s_pitem[pr];
                    t = meta >> 16;
                    c = (meta >> 8) & 63u;
                    slot = meta & 255u;
                    wc[q] = (meta >> 14) & 1u;
                } else {
                    while (s_item0[pr + 1] <= it) pr++;
                    t = pr;
                    const TableDev &tab = T.t[t];
                    const u32 cnt = s_tcnt[t], rem = it - s_item0[t];
                    c = rem / cnt;
                    j = rem - c * cnt;
                    wc[q] = col_wide(tab, c);
                    slot = c + (u32)__popcll(c ? (tab.wide & ((1ull << c) - 1ull)) : 0ull);  // payload slot of column c
                }
                const u32 e = s_toff[t] + j;
                const int32_t *src = b.payload + s_off[e] + slot;
                v[q] = wc[q] ? (long long)(((u64)(u32)src[1] << 32) | (u64)(u32)src[0]) : (long long)src[0];
                if (s_lc[e] == c) v[q] = s_lv[e];
                if (LTP_IN_BOUNDS(ctr, s_base[t] + j, T.t[t].rows_cap)) {
                    if constexpr (DESC) dst[q] = s_pdst[pr] + (u64)j * (wc[q] ? 8ull : 4ull);
                    else dst[q] = T.t[t].data + col_off(T.t[t], c) + (s_base[t] + j) * (wc[q] ? 8ull : 4ull);
                }
            }
#pragma unroll
            for (int q = 0; q < U; q++)
                if (dst[q]) store_cell(dst[q], wc[q], v[q]);
        }
        __syncthreads();
    }
}

__global__ void __launch_bounds__(kInsBlock) k_insert(BatchDev b, TablesDev T, Scratch s, Counters *ctr, int prefixed) {
    pdl_begin();
    phase_insert<kInsBlock, true>(b, T, s, ctr, prefixed != 0);
}

// Ordered rule: every insert commits, so the rank of an insert among its
// table's inserts is known once mark has counted them per insert tile.  One
// block turns the counts into exclusive prefixes in place, table by table
// (thread j scans a run of consecutive tiles), so the insert kernel needs no
// look-back across tiles.
constexpr u32 kInsPrefixBlock = 1024;
__global__ void __launch_bounds__(kInsPrefixBlock) k_ins_prefix(BatchDev b, TablesDev T, Scratch s, Counters *ctr) {
    pdl_begin();
    if (block_err(ctr)) return;
    const u64 tiles = (b.n_ops + kInsTile - 1) / kInsTile;
    const u64 per = (tiles + kInsPrefixBlock - 1) / kInsPrefixBlock;
    const u64 t0 = (u64)threadIdx.x * per, t1 = min(t0 + per, tiles);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    __shared__ u32 s_wsum[kInsPrefixBlock / 32];
    for (u32 tb = 0; tb < T.n; tb++) {
        if (!ctr->ins_total[tb]) continue;  // the same for every thread
        u32 sum = 0;
        for (u64 t = t0; t < t1; t++) sum += s.ins_pre[t * LTP_MAX_TABLES + tb];
        u32 incl = sum;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const u32 v = __shfl_up_sync(FULL_MASK, incl, d);
            if (lane >= d) incl += v;
        }
        if (lane == 31) s_wsum[warp] = incl;
        __syncthreads();
        u32 pre = incl - sum;
        for (int i = 0; i < warp; i++) pre += s_wsum[i];
        for (u64 t = t0; t < t1; t++) {
            const u32 c = s.ins_pre[t * LTP_MAX_TABLES + tb];
            s.ins_pre[t * LTP_MAX_TABLES + tb] = pre;
            pre += c;
        }
        __syncthreads();  // s_wsum is reused by the next table
    }
}

// ============================================================================
// finish: return the scratch to its clean state, count commits
// ============================================================================
template <int WB>
__device__ __forceinline__ void phase_finish(const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr,
                                             int rule) {
    const u64 gsz = (u64)gridDim.x * blockDim.x, g0 = (u64)blockIdx.x * blockDim.x + threadIdx.x;
    u32 any_ins = 0;
    for (u32 k = 0; k < T.n; k++) any_ins |= ctr->ins_total[k];
    if (blockIdx.x == 0 && threadIdx.x < T.n && !ctr->err) T.rows_now[threadIdx.x] += ctr->ins_committed[threadIdx.x];
    if (any_ins) {
        const u64 t_ins = (b.n_ops + kInsTile - 1) / kInsTile;
        for (u64 j = g0; j < t_ins * LTP_MAX_TABLES; j += gsz) {
            s.st_ins[j] = 0;
            s.ins_pre[j] = 0;
        }
    }
    const u64 ntw = ctr->n_tw;
    const bool dense = ids_dense(ctr);
    const u64 nw = Wd<WB>::n_words(s);
    if (dense) {
        // every word of the touched range: the next batch's mark finds the
        // cleared lines in L2, kept there by the evict-last hint (Zipf mark
        // 0.270 -> 0.263 ms; evict-first instead: 0.303 ms)
        const u64 pol_keep = pol_evict_last();
        const u64 whi = min(touched_hi(ctr), nw);
        for (u64 j = touched_lo(ctr) + g0; j < whi; j += gsz) Wd<WB>::clear_hint(s, j, pol_keep);
    } else {
        for (u64 j = g0; j < ntw; j += gsz)
            if (LTP_IN_BOUNDS(ctr, s.tw_list[j], nw)) Wd<WB>::clear(s, s.tw_list[j]);
    }
    // the compact views of the words that held contended cells, found
    // through the contended cells themselves
    const u64 M = ctr->M;
    for (u64 m = g0; m < M; m += gsz) {
        if (!LTP_IN_BOUNDS(ctr, m, s.cap_ops)) continue;
        const u64 w = (s.dcell[m] & ~(1ull << 63)) >> Wd<WB>::kShift;
        if (LTP_IN_BOUNDS(ctr, w, nw)) Wd<WB>::clear_view(s, w);
    }
    const u64 nc = ctr->n_c;
    const u64 t_apply = (nc + kApplyTile - 1) / kApplyTile;
    for (u64 j = g0; j < t_apply; j += gsz) s.st_apply[j] = 0;
    const int passes = sort_passes_dev(ctr->M);
    if (passes > 0) {
        u32 *st = ((passes - 1) & 1) ? s.st_sort[1] : s.st_sort[0];  // select: see phase_apply
        const u64 t_sort = (nc + kSortTile - 1) / kSortTile;
        for (u64 j = g0; j < t_sort * 256; j += gsz) st[j] = 0;
    }
    if (rule != LTP_RULE_PRIORITY) {  // classify's look-back slots (any tiling: at most one per kMinTile ops)
        const u64 t_cls = (b.n_ops + kMinTile - 1) / kMinTile;
        for (u64 j = g0; j < t_cls; j += gsz) s.st_cls[j] = 0;
    }
    if (rule == LTP_RULE_PRIORITY) {
        u32 c = 0;
        for (u64 t = g0; t < b.n_txns; t += gsz) c += b.commit[t];
        c = __reduce_add_sync(FULL_MASK, c);
        if ((threadIdx.x & 31) == 0 && c) atomicAdd(&ctr->committed, (u64)c);
    }
}

template <int WB>
__global__ void __launch_bounds__(256) k_finish(BatchDev b, TablesDev T, Scratch s, Counters *ctr, int rule) {
    pdl_begin();
    phase_finish<WB>(b, T, s, ctr, rule);
}

__global__ void k_stall(Counters *ctr, u32 ms) {
    const u64 t0 = gtimer();
    const u64 lim = (u64)ms * 1000000ull;
    volatile u32 *flag = &ctr->stall;
    while (*flag == 0u) {
        if (gtimer() - t0 > lim) {
            set_err(ctr, LTP_E_TIMEOUT);
            return;
        }
        __nanosleep(1000);
    }
}

// int64 columns hold the same seeded int32 value, sign-extended
__global__ void k_fill_seeded(TableDev t, u64 seed) {
    const u64 base = mix64(seed ^ 0x5441424C45ull);
    const u64 total = t.n_rows * t.n_cols;
    for (u64 j = (u64)blockIdx.x * blockDim.x + threadIdx.x; j < total; j += (u64)gridDim.x * blockDim.x) {
        const u64 col = j / t.n_rows, row = j - col * t.n_rows;
        const bool wc = col_wide(t, (u32)col);
        store_cell(t.data + col_off(t, (u32)col) + row * (wc ? 8ull : 4ull), wc,
                   (long long)(int32_t)(u32)mix64(base + row * t.n_cols + col));
    }
}

// out64 of the ops on int32 cells, which the execution kernels leave to
// this step: their value, sign-extended from out.
__global__ void k_widen_out(BatchDev b, TablesDev T) {
    for (u64 i = (u64)blockIdx.x * blockDim.x + threadIdx.x; i < b.n_ops; i += (u64)gridDim.x * blockDim.x) {
        const u32 w = b.opw[i], tb = opw_table(w);
        if (opw_kind(w) > LTP_OP_ADD || tb >= T.n || col_wide(T.t[tb], opw_col(w))) continue;
        b.out64[i] = (long long)b.out[i];
    }
}

__global__ void k_expand_op_txn(const u32 *txn_first, u64 n_txns, u32 *op_txn) {
    for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < n_txns; t += (u64)gridDim.x * blockDim.x)
        for (u32 i = txn_first[t]; i < txn_first[t + 1]; i++) op_txn[i] = (u32)t;
}

// The same for a txn_first that only the device has seen (no host check):
// it must start at 0, never decrease and end at n_ops.  A violation records
// LTP_E_BADARG -- every later kernel of the batch then exits at its first
// error check -- and no entry outside op_txn[0, n_ops) is written.
__global__ void k_expand_op_txn_checked(const u32 *txn_first, u64 n_txns, u64 n_ops, u32 *op_txn, Counters *ctr) {
    for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < n_txns; t += (u64)gridDim.x * blockDim.x) {
        const u64 a = txn_first[t], e = txn_first[t + 1];
        if ((t == 0 && a != 0) || e < a || (t + 1 == n_txns && e != n_ops)) set_err(ctr, LTP_E_BADARG);
        const u64 hi = e < n_ops ? e : n_ops;
        for (u64 i = a; i < hi; i++) op_txn[i] = (u32)t;
    }
}

// ============================================================================
// host-side launch plans
// ============================================================================
template <typename K>
static int occ_grid(K kernel, int block, int num_sms, size_t dyn_smem = 0) {
    int per_sm = 0;
    if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kernel, block, dyn_smem) != cudaSuccess) {
        (void)cudaGetLastError();
        per_sm = 1;
    }
    if (per_sm < 1) per_sm = 1;
    return per_sm * num_sms;
}

// Launches a batch kernel, with programmatic stream serialization when `pdl`
// (see pdl_begin): it may start while its predecessor on the stream drains.
// Stream launches use it; captured graphs do not (their launches already
// follow each other closely, and measured no faster with it).
template <typename... KP, typename... A>
static cudaError_t launch_k(bool pdl, void (*kernel)(KP...), unsigned grid, unsigned block, size_t smem,
                            cudaStream_t st, A... args) {
    cudaLaunchConfig_t c = {};
    c.gridDim = dim3(grid);
    c.blockDim = dim3(block);
    c.dynamicSmemBytes = smem;
    c.stream = st;
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    c.attrs = at;
    c.numAttrs = pdl ? 1 : 0;
    return cudaLaunchKernelEx(&c, kernel, static_cast<KP>(args)...);
}

template <int BLOCK, int IPT, int WB>
struct Front {
    static int g_mark, g_cls, sms;
    static constexpr size_t kMarkSmem = mark_smem_bytes<BLOCK, IPT, WB>();
    static void grids(int num_sms) {
        if (sms != num_sms) {
            if (cudaFuncSetAttribute(k_mark<BLOCK, IPT, WB>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     (int)kMarkSmem) != cudaSuccess)
                return;  // the launch below then reports the error
            g_mark = occ_grid(k_mark<BLOCK, IPT, WB>, BLOCK, num_sms, kMarkSmem);
            g_cls = occ_grid(k_classify<BLOCK, IPT, WB>, BLOCK, num_sms);
            sms = num_sms;
        }
    }
    static cudaError_t mark(const Launch &L, const BatchDev &b, const TablesDev &T, const Scratch &s, Counters *ctr) {
        grids(L.num_sms);
        const u64 tiles = (b.n_ops + (u64)BLOCK * IPT - 1) / ((u64)BLOCK * IPT);
        const int g = (int)(tiles < (u64)g_mark ? (tiles ? tiles : 1) : (u64)g_mark);
        return launch_k(L.pdl, k_mark<BLOCK, IPT, WB>, g, BLOCK, kMarkSmem, L.stream, b, T, s, ctr);
    }
    static cudaError_t classify(const Launch &L, const BatchDev &b, const TablesDev &T, const Scratch &s,
                                Counters *ctr) {
        grids(L.num_sms);
        const u64 tiles = (b.n_ops + (u64)BLOCK * IPT - 1) / ((u64)BLOCK * IPT);
        const int g = (int)(tiles < (u64)g_cls ? (tiles ? tiles : 1) : (u64)g_cls);
        return launch_k(L.pdl, k_classify<BLOCK, IPT, WB>, g, BLOCK, 0, L.stream, b, T, s, ctr);
    }
};
template <int BLOCK, int IPT, int WB> int Front<BLOCK, IPT, WB>::g_mark = 0;
template <int BLOCK, int IPT, int WB> int Front<BLOCK, IPT, WB>::g_cls = 0;
template <int BLOCK, int IPT, int WB> int Front<BLOCK, IPT, WB>::sms = 0;

typedef cudaError_t (*front_fn)(const Launch &, const BatchDev &, const TablesDev &, const Scratch &, Counters *);

// 64-cell words exist for the tilings whose mark hash (28 B per slot) fits a
// block's shared memory: up to 2,048 ops per tile
bool tiling_supported(int block, int ipt, int word_bits) {
    const bool known = (block == 128 || block == 256 || block == 512) && (ipt == 1 || ipt == 2 || ipt == 4 || ipt == 8);
    return known && (word_bits == 32 || (word_bits == 64 && block * ipt <= 2048));
}

static void pick_front(const Tuning &t, front_fn *mark, front_fn *classify) {
#define LTP_FRONT(B, I, W)                                     \
    if (t.block == B && t.ipt == I && t.word_bits == W) {      \
        *mark = Front<B, I, W>::mark;                          \
        *classify = Front<B, I, W>::classify;                  \
        return;                                                \
    }
    LTP_FRONT(128, 1, 32) LTP_FRONT(128, 2, 32) LTP_FRONT(128, 4, 32) LTP_FRONT(128, 8, 32)
    LTP_FRONT(256, 1, 32) LTP_FRONT(256, 2, 32) LTP_FRONT(256, 4, 32) LTP_FRONT(256, 8, 32)
    LTP_FRONT(512, 1, 32) LTP_FRONT(512, 2, 32) LTP_FRONT(512, 4, 32) LTP_FRONT(512, 8, 32)
    LTP_FRONT(128, 1, 64) LTP_FRONT(128, 2, 64) LTP_FRONT(128, 4, 64) LTP_FRONT(128, 8, 64)
    LTP_FRONT(256, 1, 64) LTP_FRONT(256, 2, 64) LTP_FRONT(256, 4, 64) LTP_FRONT(256, 8, 64)
    LTP_FRONT(512, 1, 64) LTP_FRONT(512, 2, 64) LTP_FRONT(512, 4, 64)
#undef LTP_FRONT
    *mark = Front<256, 4, 32>::mark;
    *classify = Front<256, 4, 32>::classify;
}

static int capped(int grid, u64 upper) { return (int)((u64)grid < upper ? (u64)grid : (upper ? upper : 1)); }

cudaError_t launch_execute(const Launch &L_in, const BatchDev &b_in, const TablesDev &T, const Scratch &s,
                           Counters *ctr) {
    TraceRange tr("launch batch kernels");
    Launch L = L_in;
    BatchDev b = b_in;
    b.flags = L.tune.flags;
    (void)cudaGetLastError();  // report only the launches below
    // stage event i is recorded after kernel i; event 0 of the batch precedes everything
    // under stream capture the stage events become external event nodes, so
    // they still carry timestamps when the graph replays
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(L.stream, &cap);
    // dependent launch for stream launches, and inside captured graphs for
    // small batches only (measured: a gain for batches of a few thousand
    // transactions, a loss at 2^16 x 10 ops and above)
    L.pdl = cap != cudaStreamCaptureStatusActive || b_in.n_ops < (1ull << 18);
    const unsigned ev_flags = cap == cudaStreamCaptureStatusActive ? cudaEventRecordExternal : cudaEventRecordDefault;
    auto mark_ev = [&](int i) {
        if (L.timing) cudaEventRecordWithFlags(L.ev[i], L.stream, ev_flags);
        if (L.progress && i == L.progress_stage) cudaEventRecordWithFlags(L.progress, L.stream, ev_flags);
    };
    mark_ev(0);
    if (L.stall) k_stall<<<1, 1, 0, L.stream>>>(ctr, L.stall_ms);
    front_fn f_mark, f_cls;
    pick_front(L.tune, &f_mark, &f_cls);
    // conflict-word width of every kernel of the batch (an unsupported tiling
    // falls back to 256 x 4 with 32-cell words in pick_front)
    const bool wide_words = L.tune.word_bits == 64 && tiling_supported(L.tune.block, L.tune.ipt, 64);
    cudaError_t le = cudaSuccess;  // the first failed launch
    auto chk = [&](cudaError_t e) {
        if (le == cudaSuccess) le = e;
    };
    chk(f_mark(L, b, T, s, ctr));
    mark_ev(1);
    {
        static int gi = 0, sms = 0;
        if (sms != L.num_sms) {
            gi = occ_grid(k_ids<32>, kIdsBlock, L.num_sms);
            sms = L.num_sms;
        }
        const int g = capped(gi, (b.n_ops + kIdsTile - 1) / kIdsTile);
        chk(launch_k(L.pdl, wide_words ? k_ids<64> : k_ids<32>, g, kIdsBlock, 0, L.stream, T, s, ctr));
        chk(launch_k(L.pdl, k_dbase, L.num_sms * 8, 256, 0, L.stream, T, s, ctr, (int)(L.rule == LTP_RULE_PRIORITY)));
    }
    mark_ev(2);
    const int gstream = L.num_sms * 8;
    if (L.rule != LTP_RULE_PRIORITY) {
        chk(f_cls(L, b, T, s, ctr));
        mark_ev(3);
        static int gs = 0, ga = 0, sms = 0;
        if (sms != L.num_sms) {
            gs = occ_grid(k_sort_pass<0>, kSortBlock, L.num_sms);
            ga = occ_grid(k_apply_auto, kApplyBlock, L.num_sms);
            sms = L.num_sms;
        }
        const int gsort = capped(gs, (b.n_ops + kSortTile - 1) / kSortTile);
        // at most n_ops contended ids: passes beyond their width are not launched
        int max_passes = 1;
        while (max_passes < 4 && ((b.n_ops - 1) >> (8 * max_passes)) != 0) max_passes++;
        chk(launch_k(L.pdl, k_sort_pass<0>, gsort, kSortBlock, 0, L.stream, s, ctr, b.n_ops));
        mark_ev(4);
        if (max_passes > 1) chk(launch_k(L.pdl, k_sort_pass<1>, gsort, kSortBlock, 0, L.stream, s, ctr, b.n_ops));
        mark_ev(5);
        if (max_passes > 2) chk(launch_k(L.pdl, k_sort_pass<2>, gsort, kSortBlock, 0, L.stream, s, ctr, b.n_ops));
        mark_ev(6);
        if (max_passes > 3) chk(launch_k(L.pdl, k_sort_pass<3>, gsort, kSortBlock, 0, L.stream, s, ctr, b.n_ops));
        mark_ev(7);
        const int gapp = capped(ga, (b.n_ops + kApplyTile - 1) / kApplyTile);
        chk(launch_k(L.pdl, T.any_wide ? k_apply_auto : k_apply<u32>, gapp, kApplyBlock, 0, L.stream, b, T, s, ctr));
        mark_ev(8);
    } else {
        chk(launch_k(L.pdl, wide_words ? k_r1_minw<64> : k_r1_minw<32>, gstream, 256, 0, L.stream, b, T, s, ctr));
        mark_ev(3);
        chk(launch_k(L.pdl, wide_words ? k_r1_abort<64> : k_r1_abort<32>, gstream, 256, 0, L.stream, b, T, s, ctr));
        mark_ev(4);
        chk(launch_k(L.pdl, wide_words ? k_r1_exec<64> : k_r1_exec<32>, gstream, 256, 0, L.stream, b, T, s, ctr));
        for (int i = 5; i <= 8; i++) mark_ev(i);
    }
    {
        static int gins = 0, sms = 0;
        if (sms != L.num_sms) {
            chk(cudaFuncSetAttribute(k_insert, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kInsSmemDesc));
            gins = occ_grid(k_insert, kInsBlock, L.num_sms, kInsSmemDesc);
            sms = L.num_sms;
        }
        if (b.payload_len) {  // a batch without payload has no valid insert
            const int prefixed = L.rule != LTP_RULE_PRIORITY;
            if (prefixed) chk(launch_k(L.pdl, k_ins_prefix, 1, kInsPrefixBlock, 0, L.stream, b, T, s, ctr));
            chk(launch_k(L.pdl, k_insert, capped(gins, (b.n_ops + kInsTile - 1) / kInsTile), kInsBlock, kInsSmemDesc,
                         L.stream, b, T, s, ctr, prefixed));
        }
    }
    mark_ev(9);
    chk(launch_k(L.pdl, wide_words ? k_finish<64> : k_finish<32>, gstream, 256, 0, L.stream, b, T, s, ctr, L.rule));
    mark_ev(10);
    const cudaError_t e = cudaGetLastError();
    return le != cudaSuccess ? le : e;
}

// ============================================================================
// persistent fused kernel: one cooperative launch runs a list of batches
// through every phase (bitmap build -> ids -> classify -> sort -> apply ->
// inserts -> clean-up) with grid-wide barriers in between and no host round
// trip.  Each barrier is a bounded spin; a timeout or any device error ends
// the run for every block.
// ============================================================================
__device__ __forceinline__ void grid_sync(u32 *bar, u32 nblocks, Counters *ctr) {
    __syncthreads();
    if (threadIdx.x == 0) {
        const u32 gen = ld_acquire32(bar + 1);
        __threadfence();
        const u32 arrived = atomicAdd(bar, 1u);
        if (arrived == nblocks - 1) {
            bar[0] = 0;
            __threadfence();
            st_release32(bar + 1, gen + 1);
        } else {
            const u64 t0 = gtimer();
            volatile int *err = &ctr->err;
            while (ld_acquire32(bar + 1) == gen) {
                if (*err) break;
                if (gtimer() - t0 > kSpinLimitNs) {
                    set_err(ctr, LTP_E_TIMEOUT);
                    break;
                }
                __nanosleep(32);
            }
        }
    }
    __syncthreads();
}

struct PersistArgs {
    const BatchDev *batches;
    Counters *const *snaps;  // [n_batches] where each batch's counters go after it ran
    u32 n_batches;
    int rule;
    TablesDev T;
    Scratch s;
    Counters *ctr;
    u32 *bar;  // [2] barrier arrival count and generation
};

constexpr int kPBlock = 256, kPIpt = 4;
// dynamic shared memory of the persistent kernel: the larger of the mark
// phase's hash (4 arrays of 2 x tile words) and the insert staging
constexpr size_t kPersistSmem = 4ull * 2 * kPBlock * kPIpt * sizeof(u32) > kInsSmem
                                    ? 4ull * 2 * kPBlock * kPIpt * sizeof(u32) : (size_t)kInsSmem;

__global__ void __launch_bounds__(kPBlock, 2) k_persist(PersistArgs a) {
    const u32 nb = gridDim.x;
    for (u32 j = 0; j < a.n_batches; j++) {
        const BatchDev b = a.batches[j];
        if (blockIdx.x == 0) {  // fresh counters; a device error stays sticky for the run
            const int keep = a.ctr->err;
            __syncthreads();
            u32 *w = reinterpret_cast<u32 *>(a.ctr);
            for (u32 i = threadIdx.x; i < sizeof(Counters) / 4; i += blockDim.x) w[i] = 0u;
            __syncthreads();
            if (threadIdx.x == 0) a.ctr->err = keep;
        }
        for (u64 t = (u64)blockIdx.x * blockDim.x + threadIdx.x; t < b.n_txns; t += (u64)nb * blockDim.x) b.commit[t] = 1;
        grid_sync(a.bar, nb, a.ctr);
        if (block_err(a.ctr)) break;
        phase_mark<kPBlock, kPIpt, 32>(b, a.T, a.s, a.ctr);
        grid_sync(a.bar, nb, a.ctr);
        phase_ids<kPBlock, 32>(a.T, a.s, a.ctr);
        grid_sync(a.bar, nb, a.ctr);
        phase_dbase(a.T, a.s, a.ctr, a.rule == LTP_RULE_PRIORITY);
        grid_sync(a.bar, nb, a.ctr);
        if (a.rule != LTP_RULE_PRIORITY) {
            phase_classify<kPBlock, kPIpt, 32>(b, a.T, a.s, a.ctr);
            grid_sync(a.bar, nb, a.ctr);
            // only the passes the contended ids need (M is the same for every
            // block after the barrier, so every block skips the same ones)
            const int passes = sort_passes_dev(*(volatile u32 *)&a.ctr->M);
            for (int P = 0; P < passes; P++) {
                phase_sort_pass<kPBlock>(P, a.s, a.ctr, b.n_ops);
                grid_sync(a.bar, nb, a.ctr);
            }
            if (a.T.any_wide && *(volatile u32 *)&a.ctr->wide_ops) phase_apply<kPBlock, u64>(b, a.T, a.s, a.ctr);
            else phase_apply<kPBlock, u32>(b, a.T, a.s, a.ctr);
        } else {
            phase_r1_minw<32>(b, a.T, a.s, a.ctr);
            grid_sync(a.bar, nb, a.ctr);
            phase_r1_abort<32>(b, a.T, a.s, a.ctr);
            grid_sync(a.bar, nb, a.ctr);
            phase_r1_exec<32>(b, a.T, a.s, a.ctr);
        }
        grid_sync(a.bar, nb, a.ctr);
        if (b.payload_len) {  // a batch without payload has no valid insert
            phase_insert<kPBlock, false>(b, a.T, a.s, a.ctr, false);
            grid_sync(a.bar, nb, a.ctr);
        }
        phase_finish<32>(b, a.T, a.s, a.ctr, a.rule);
        grid_sync(a.bar, nb, a.ctr);
        if (blockIdx.x == 0) {
            const u32 *src = reinterpret_cast<const u32 *>(a.ctr);
            u32 *dst = reinterpret_cast<u32 *>(a.snaps[j]);
            for (u32 i = threadIdx.x; i < sizeof(Counters) / 4; i += blockDim.x) dst[i] = src[i];
        }
        if (block_err(a.ctr)) break;
        grid_sync(a.bar, nb, a.ctr);
    }
}

cudaError_t launch_persistent(cudaStream_t st, int num_sms, int rule, const BatchDev *d_batches,
                              Counters *const *d_snaps, u32 n_batches, const TablesDev &T, const Scratch &s,
                              Counters *ctr, u32 *bar) {
    constexpr size_t smem = kPersistSmem;
    static int grid = 0, sms = 0;
    if (sms != num_sms) {
        cudaError_t fe = cudaFuncSetAttribute(k_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (fe != cudaSuccess) return fe;
        grid = occ_grid(k_persist, kPBlock, num_sms, smem);
        sms = num_sms;
    }
    (void)cudaGetLastError();
    cudaError_t e = cudaMemsetAsync(bar, 0, 2 * sizeof(u32), st);
    if (e != cudaSuccess) return e;
    PersistArgs a;
    a.batches = d_batches;
    a.snaps = d_snaps;
    a.n_batches = n_batches;
    a.rule = rule;
    a.T = T;
    a.s = s;
    a.ctr = ctr;
    a.bar = bar;
    void *args[] = {&a};
    return cudaLaunchCooperativeKernel((const void *)k_persist, dim3(grid), dim3(kPBlock), args, smem, st);
}

int persistent_grid(int num_sms) {
    constexpr size_t smem = kPersistSmem;
    cudaFuncSetAttribute(k_persist, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    return occ_grid(k_persist, kPBlock, num_sms, smem);
}

cudaError_t launch_reset_scratch(cudaStream_t st, const Scratch &s) {
    cudaMemsetAsync(s.words, 0, (s.n_words + 1) * sizeof(WordState), st);  // + the 64-cell layout's spare entry
    cudaMemsetAsync(s.cview, 0, (s.n_words + 1) * sizeof(uint2), st);
    cudaMemsetAsync(s.st_sort[0], 0, s.cap_sort_tiles * 256 * 4, st);
    cudaMemsetAsync(s.st_sort[1], 0, s.cap_sort_tiles * 256 * 4, st);
    cudaMemsetAsync(s.st_cls, 0, s.cap_tiles * 8, st);
    cudaMemsetAsync(s.st_apply, 0, s.cap_tiles * 8, st);
    cudaMemsetAsync(s.st_ins, 0, s.cap_tiles * LTP_MAX_TABLES * 4, st);
    if (s.ins_pre != s.st_ins) cudaMemsetAsync(s.ins_pre, 0, s.cap_tiles * LTP_MAX_TABLES * 4, st);
    return cudaGetLastError();
}

cudaError_t launch_fill_seeded(cudaStream_t st, const TableDev &t, u64 seed) {
    k_fill_seeded<<<1024, 256, 0, st>>>(t, seed);
    return cudaGetLastError();
}

__global__ void k_set_u64(u64 *dst, u64 value) { *dst = value; }

cudaError_t launch_set_u64(cudaStream_t st, u64 *dst, u64 value) {
    k_set_u64<<<1, 1, 0, st>>>(dst, value);
    return cudaGetLastError();
}

cudaError_t launch_widen_out(cudaStream_t st, const BatchDev &b, const TablesDev &T) {
    if (b.n_ops == 0 || !b.out64) return cudaSuccess;
    u64 blocks = (b.n_ops + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_widen_out<<<(unsigned)blocks, 256, 0, st>>>(b, T);
    return cudaGetLastError();
}

cudaError_t launch_expand_op_txn(cudaStream_t st, const u32 *txn_first, u64 n_txns, u32 *op_txn) {
    if (n_txns == 0) return cudaSuccess;
    u64 blocks = (n_txns + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_expand_op_txn<<<(unsigned)blocks, 256, 0, st>>>(txn_first, n_txns, op_txn);
    return cudaGetLastError();
}

cudaError_t launch_expand_op_txn_checked(cudaStream_t st, const u32 *txn_first, u64 n_txns, u64 n_ops, u32 *op_txn,
                                         Counters *ctr) {
    if (n_txns == 0) return cudaSuccess;
    u64 blocks = (n_txns + 255) / 256;
    if (blocks > 4096) blocks = 4096;
    k_expand_op_txn_checked<<<(unsigned)blocks, 256, 0, st>>>(txn_first, n_txns, n_ops, op_txn, ctr);
    return cudaGetLastError();
}

}  // namespace ltp
