// group_id_i64 and group_id2_i64_i64: dense ids numbered by first occurrence
// (src/kernels/scalar/group.rs:207-301).
//
// The ids depend only on the order in which distinct keys first appear (group.rs:1-5), so any
// correct table gives the reference's output. Two kernels:
//  1. insert: open addressing with linear probing. A free slot holds the key EMPTY (the byte
//     0x80 repeated) and is claimed by a CAS on the key itself (a 128-bit CAS for key pairs),
//     so a probe that reads its key needs no further synchronisation. Slot 0 is never probed:
//     it belongs to the key EMPTY (or the pair (EMPTY, EMPTY)), whose rows go there directly.
//     Each slot keeps the smallest row that holds its key (atomicMin, skipped when the stored
//     row is already smaller), and each row records its slot. A thread probes four rows at once.
//  2. number: a row is a first occurrence when its slot's smallest row is itself; a
//     decoupled-lookback compaction over rows gives each first occurrence its rank, which is
//     the group's id, stored in the slot; the same kernel writes every row's id.
// Table size: the reference's maximum is nextpow2(2n) slots (group.rs:226-229). When that is
// above the first table's size (2^group_first_table_log2 slots from the autotuner's table,
// 2^21 by default, which stays in L2), the insert first runs on that table; it gives up (an
// overflow flag) once half its slots hold keys or a probe of 64 slots is reached, and only then
// is the full table filled. Inputs with few distinct keys never touch the large table.
#include "lookback.cuh"
#include "reduce_common.h"

namespace vkc {

constexpr int GI_THREADS = 256;
constexpr int GI_ITEMS = 16;
constexpr int GI_TILE = GI_THREADS * GI_ITEMS;
constexpr int GI_ROWS = 4;  // rows a thread probes at once
constexpr unsigned long long GI_EMPTY = 0x8080808080808080ull;
constexpr unsigned GI_SMALL_PROBES = 64;

// A slot is one 16-byte record (key, smallest row, id), or 32 bytes for key pairs (key a,
// key b, smallest row, id, unused), so the probe, the claim and the row update of a key touch
// one line of the table.
struct GroupTable {
    unsigned long long *words;  // W words per slot: the key (two for pairs, GI_EMPTY when free),
                                // then uint2 {x = smallest row of the key, y = group id}
    unsigned long long mask;    // slots - 1
    int w;                      // words per slot: 2, or 4 for key pairs
    __device__ __forceinline__ uint2 *meta(unsigned long long s) const {
        return reinterpret_cast<uint2 *>(words + w * s + (w == 4 ? 2 : 1));
    }
};

// group.rs:40-47 (mix) with a fixed odd multiplier; the ids do not depend on it.
__device__ __forceinline__ unsigned long long gmix(unsigned long long x) {
    return (x ^ (x >> 32)) * 0x9E3779B97F4A7C15ull;
}

__device__ __forceinline__ unsigned long long gi_first(unsigned long long h, unsigned long long mask) {
    const unsigned long long s = (h >> 32 ^ h) & mask;
    return s ? s : 1ull;
}

__device__ __forceinline__ unsigned long long gi_next(unsigned long long s, unsigned long long mask) {
    s = (s + 1) & mask;
    return s ? s : 1ull;
}

__device__ __forceinline__ void ld_relaxed_pair(const unsigned long long *p, unsigned long long &a,
                                                unsigned long long &b) {
    asm volatile("ld.relaxed.gpu.global.v2.u64 {%0, %1}, [%2];" : "=l"(a), "=l"(b) : "l"(p) : "memory");
}

// 128-bit compare-and-swap of the pair at p (16-byte aligned): returns the old pair.
__device__ __forceinline__ void cas_pair(unsigned long long *p, unsigned long long ca, unsigned long long cb,
                                         unsigned long long na, unsigned long long nb, unsigned long long &oa,
                                         unsigned long long &ob) {
    asm volatile(
        "{\n\t.reg .b128 c, v, o;\n\t"
        "mov.b128 c, {%2, %3};\n\t"
        "mov.b128 v, {%4, %5};\n\t"
        "atom.relaxed.gpu.global.cas.b128 o, [%6], c, v;\n\t"
        "mov.b128 {%0, %1}, o;\n\t}"
        : "=l"(oa), "=l"(ob)
        : "l"(ca), "l"(cb), "l"(na), "l"(nb), "l"(p)
        : "memory");
}

__device__ __forceinline__ unsigned ld_relaxed32(const unsigned *p) {
    unsigned v;
    asm volatile("ld.relaxed.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// SMALL: the attempt on the small table, which gives up through flags[1] (flags[0] counts the
// distinct keys inserted). Otherwise the table has room for every key and a probe longer than
// the table only records a timeout. Probes read the slot first and claim a free one by CAS,
// except for single keys on the full table (many distinct keys): there one 128-bit CAS both
// reads the slot and claims it with the row as its smallest row.
template <bool PAIR, bool SMALL>
__global__ void __launch_bounds__(GI_THREADS) gi_insert_kernel(const long long *__restrict__ a,
                                                               const long long *__restrict__ b, int64_t n,
                                                               GroupTable t, unsigned *__restrict__ slot_of,
                                                               unsigned *flags, DevStatus *st) {
    constexpr bool CAS_FIRST = !SMALL && !PAIR;
    const int lane = threadIdx.x & 31;
    const int64_t step = static_cast<int64_t>(gridDim.x) * GI_THREADS * GI_ROWS;
    // The full table always has a free slot, so a probe ends within `mask` steps.
    const unsigned long long limit = SMALL ? GI_SMALL_PROBES : t.mask;
    const unsigned max_keys = static_cast<unsigned>((t.mask + 1) / 2);
    for (int64_t base = static_cast<int64_t>(blockIdx.x) * GI_THREADS * GI_ROWS; base < n; base += step) {
        if (SMALL) {
            unsigned ov = lane == 0 ? ld_relaxed32(flags + 1) : 0u;
            if (__shfl_sync(FULL, ov, 0)) return;  // the whole warp leaves together
        }
        unsigned long long ka[GI_ROWS], kb[GI_ROWS], s[GI_ROWS];
        unsigned cur[GI_ROWS];  // the slot's smallest row as last seen (CAS_FIRST)
        unsigned pend = 0, in = 0, fresh = 0;
        bool gave_up = false;
#pragma unroll
        for (int j = 0; j < GI_ROWS; ++j) {
            const int64_t r = base + j * GI_THREADS + threadIdx.x;
            ka[j] = kb[j] = GI_EMPTY;
            s[j] = 0;
            cur[j] = 0xffffffffu;
            if (r < n) {
                in |= 1u << j;
                ka[j] = static_cast<unsigned long long>(__ldcs(a + r));
                if (PAIR) kb[j] = static_cast<unsigned long long>(__ldcs(b + r));
                if (ka[j] != GI_EMPTY || (PAIR && kb[j] != GI_EMPTY)) {
                    s[j] = gi_first(PAIR ? gmix(gmix(ka[j]) ^ kb[j]) : gmix(ka[j]), t.mask);
                    pend |= 1u << j;
                }
            }
        }
        unsigned long long probes = 0;
        while (pend) {
            unsigned long long va[GI_ROWS], vb[GI_ROWS];
#pragma unroll
            for (int j = 0; j < GI_ROWS; ++j) {
                va[j] = vb[j] = 0;
                if (pend & (1u << j)) {
                    if (CAS_FIRST) {
                        const unsigned long long row = static_cast<unsigned long long>(base + j * GI_THREADS + threadIdx.x);
                        cas_pair(t.words + 2 * s[j], GI_EMPTY, ~0ull, ka[j], 0xffffffff00000000ull | row, va[j], vb[j]);
                    } else if (PAIR) {
                        ld_relaxed_pair(t.words + 4 * s[j], va[j], vb[j]);
                    } else {
                        va[j] = ld_relaxed64(t.words + 2 * s[j]);
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < GI_ROWS; ++j) {
                if (!(pend & (1u << j))) continue;
                bool done = false;
                if (CAS_FIRST) {
                    // A free slot always holds (EMPTY, all ones), so an EMPTY key means the CAS won.
                    if (va[j] == GI_EMPTY) {
                        done = true;
                        cur[j] = 0u;  // the claim stored this row
                    } else if (va[j] == ka[j]) {
                        done = true;
                        cur[j] = static_cast<unsigned>(vb[j]);
                    }
                } else if (!PAIR) {
                    if (va[j] == ka[j]) {
                        done = true;
                    } else if (va[j] == GI_EMPTY) {
                        const unsigned long long old = atomicCAS(t.words + 2 * s[j], GI_EMPTY, ka[j]);
                        if (old == GI_EMPTY) ++fresh;
                        done = old == GI_EMPTY || old == ka[j];
                    }
                } else if (va[j] != GI_EMPTY && vb[j] != GI_EMPTY) {
                    // A slot is written once, from (EMPTY, EMPTY): a pair with no EMPTY half is whole.
                    done = va[j] == ka[j] && vb[j] == kb[j];
                } else {
                    unsigned long long oa, ob;
                    cas_pair(t.words + 4 * s[j], GI_EMPTY, GI_EMPTY, ka[j], kb[j], oa, ob);
                    if (oa == GI_EMPTY && ob == GI_EMPTY) ++fresh;
                    done = (oa == GI_EMPTY && ob == GI_EMPTY) || (oa == ka[j] && ob == kb[j]);
                }
                if (done) pend &= ~(1u << j);
                else s[j] = gi_next(s[j], t.mask);
            }
            if (pend && ++probes > limit) {
                gave_up = true;
                break;
            }
        }
        if (gave_up) {
            if (SMALL) atomicExch(flags + 1, 1u);
            else set_timeout(st);
        }
        if (SMALL) {
            const unsigned c = __reduce_add_sync(FULL, fresh);
            if (lane == 0 && c && atomicAdd(flags, c) + c > max_keys) atomicExch(flags + 1, 1u);
        }
        if (gave_up) continue;
#pragma unroll
        for (int j = 0; j < GI_ROWS; ++j) {
            if (!(in & (1u << j))) continue;
            const unsigned row = static_cast<unsigned>(base + j * GI_THREADS + threadIdx.x);
            unsigned *m = &t.meta(s[j])->x;
            if ((CAS_FIRST && s[j] != 0 ? cur[j] : ld_relaxed32(m)) > row) atomicMin(m, row);
            slot_of[row] = static_cast<unsigned>(s[j]);
        }
    }
}

// Numbers the first occurrences in row order (a compaction of the rows whose slot's smallest
// row is themselves), stores each group's id in its slot, and writes every row's id. A row
// whose key first occurs in this tile takes its id from the tile's bitmap of first
// occurrences; any other key first occurs in an earlier tile, which stores the id right after
// its own lookback, so the row reads it from the slot (waiting, bounded, until it is there).
constexpr int GI_OUT_STRIDE = GI_ITEMS + 1;  // padded rows of the staged ids (bank spread)

__global__ void __launch_bounds__(GI_THREADS, 4) gi_number_kernel(const unsigned *__restrict__ slot_of, int64_t n,
                                                                  GroupTable t, int tiles, unsigned long long *words,
                                                                  unsigned epoch, unsigned *counters,
                                                                  long long *__restrict__ out, DevStatus *st) {
    __shared__ unsigned long long s_prefix;
    __shared__ unsigned s_keep[GI_TILE / 32];  // bit i of word w: row 32w + i of the tile is a first occurrence
    __shared__ unsigned s_wpre[GI_TILE / 32];  // first occurrences of the tile before word w
    __shared__ long long s_out[GI_THREADS * GI_OUT_STRIDE];
    const int tile = take_ticket(counters);
    const int64_t t0 = static_cast<int64_t>(tile) * GI_TILE;
    const int64_t row0 = t0 + threadIdx.x * GI_ITEMS;
    unsigned sl[GI_ITEMS];
    if (row0 + GI_ITEMS <= n) {
        const uint4 *v = reinterpret_cast<const uint4 *>(slot_of + row0);
#pragma unroll
        for (int q = 0; q < GI_ITEMS / 4; ++q) {
            const uint4 w = __ldcs(v + q);
            sl[4 * q] = w.x;
            sl[4 * q + 1] = w.y;
            sl[4 * q + 2] = w.z;
            sl[4 * q + 3] = w.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < GI_ITEMS; ++j) sl[j] = row0 + j < n ? slot_of[row0 + j] : 0u;
    }
    int rel[GI_ITEMS];  // the key's first row relative to the tile (negative: an earlier tile)
    unsigned keep = 0;
#pragma unroll
    for (int j = 0; j < GI_ITEMS; ++j) {
        const int64_t r = row0 + j;
        rel[j] = -1;
        if (r < n) {
            const unsigned m = t.meta(sl[j])->x;
            rel[j] = static_cast<int>(static_cast<int64_t>(m) - t0);
            if (m == static_cast<unsigned>(r)) keep |= 1u << j;
        }
    }
    const unsigned odd = __shfl_down_sync(FULL, keep, 1);
    if (!(threadIdx.x & 1)) s_keep[threadIdx.x >> 1] = keep | (odd << 16);
    unsigned long long c = __popc(keep), tile_count;
    const unsigned long long off = block_exclusive_sum<unsigned long long>(c, &tile_count);
    if (!(threadIdx.x & 1)) s_wpre[threadIdx.x >> 1] = static_cast<unsigned>(off);
    if (threadIdx.x < 32) {
        unsigned long long pre = lookback_publish<4, CountRec>(words, tile, tile_count, 0ull, epoch, st);
        if (threadIdx.x == 0) s_prefix = pre;
    }
    __syncthreads();
    const unsigned prefix = static_cast<unsigned>(s_prefix);
    unsigned id = prefix + static_cast<unsigned>(off);
#pragma unroll
    for (int j = 0; j < GI_ITEMS; ++j)
        if (keep & (1u << j)) t.meta(sl[j])->y = id++;
#pragma unroll
    for (int j = 0; j < GI_ITEMS; ++j) {
        if (row0 + j >= n) continue;
        unsigned g;
        if (rel[j] >= 0) {
            const int w = rel[j] >> 5, bit = rel[j] & 31;
            g = prefix + s_wpre[w] + __popc(s_keep[w] & ((1u << bit) - 1u));
        } else {
            const unsigned *p = &t.meta(sl[j])->y;
            unsigned it = 0;
            const unsigned limit = wait_limit(st);
            while ((g = ld_relaxed32(p)) == 0xffffffffu) {
                if (++it > limit) {
                    set_timeout(st);
                    break;
                }
                backoff(it);
            }
        }
        s_out[threadIdx.x * GI_OUT_STRIDE + j] = static_cast<long long>(g);
    }
    __syncthreads();
    const int rows = static_cast<int>(n - t0 < GI_TILE ? n - t0 : GI_TILE);
    for (int i = threadIdx.x; i < rows; i += GI_THREADS)
        __stcs(out + t0 + i, s_out[(i / GI_ITEMS) * GI_OUT_STRIDE + (i % GI_ITEMS)]);
    release_ticket(counters, tiles);
}

// Every slot free: keys GI_EMPTY, smallest row and id all ones.
__global__ void __launch_bounds__(256) gi_clear_kernel(ulonglong2 *__restrict__ p, int64_t pairs, int w) {
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const ulonglong2 key = make_ulonglong2(GI_EMPTY, w == 4 ? GI_EMPTY : ~0ull);
    const ulonglong2 rest = make_ulonglong2(~0ull, ~0ull);
    for (int64_t i = static_cast<int64_t>(blockIdx.x) * blockDim.x + threadIdx.x; i < pairs; i += stride)
        p[i] = (w == 2 || (i & 1) == 0) ? key : rest;
}

// ------------------------------------------------------------------ region-partitioned tables
//
// Many distinct keys (the first table gave up) on a large input: a table of 2n slots is far
// beyond L2, so each probe, claim and smallest-row update is a DRAM burst. Instead the rows are
// put in region order by the top GR_BITS bits of their key's hash (count per tile and region,
// one exclusive scan, a partition staged in shared memory that writes each region's runs of
// (key, row) and each row's slot in its tile's region-sorted order), and then the regions go
// through three sub-tables in rotation that stay in L2, one launch per region: a region's
// sub-table is cleared, filled (claim by 128-bit CAS, smallest row by atomicMin) and read back
// (each pair's smallest row of its key) in three consecutive launches, each of which also does
// the other two jobs for the neighbouring regions. The launches are bound by the L2's 128-bit
// CAS operations, not by DRAM: tables at load up to 2/3 (fitting L2 better) made probes longer
// and the call slower, and so did slots tagged with the region instead of cleared (a read
// before each CAS). The smallest rows go back to row order
// through the tiles' staged runs, and the numbering runs in row order as in gi_number_kernel,
// except that a row whose key first occurs in an earlier tile reads its id from the output row
// of that first occurrence (written by then, or awaited with a bounded wait).
constexpr int GR_BITS = 8, GR_NB = 1 << GR_BITS;
constexpr int GR_THREADS = 256, GR_ITEMS = 16, GR_TILE = GR_THREADS * GR_ITEMS;

__device__ __forceinline__ unsigned gr_region(unsigned long long key) {
    return static_cast<unsigned>(gmix(key) >> (64 - GR_BITS));
}

// Warp 0: exclusive prefix of GR_NB counts get(b) into s_start[0 .. GR_NB - 1], the total into
// s_start[GR_NB].
template <class Get> __device__ __forceinline__ void gr_starts(Get get, unsigned *s_start) {
    const int lane = threadIdx.x & 31;
    unsigned run = 0;
#pragma unroll
    for (int b0 = 0; b0 < GR_NB; b0 += 32) {
        const unsigned c = get(b0 + lane);
        unsigned x = c;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const unsigned y = __shfl_up_sync(FULL, x, o);
            if (lane >= o) x += y;
        }
        s_start[b0 + lane] = run + x - c;
        run += __shfl_sync(FULL, x, 31);
    }
    if (lane == 0) s_start[GR_NB] = run;
}

__device__ __forceinline__ int gr_region_of(const unsigned *s_start, unsigned v) {
    int lo = 0, hi = GR_NB;
#pragma unroll
    for (int it = 0; it < GR_BITS; ++it) {
        const int mid = (lo + hi) >> 1;
        if (s_start[mid] <= v) lo = mid;
        else hi = mid;
    }
    return lo;
}

__global__ void __launch_bounds__(GR_THREADS) gr_count_kernel(const long long *__restrict__ keys, int64_t n, int tiles,
                                                              unsigned *__restrict__ counts) {
    __shared__ unsigned h[GR_NB];
    if (threadIdx.x < GR_NB) h[threadIdx.x] = 0;
    __syncthreads();
    const int64_t base = static_cast<int64_t>(blockIdx.x) * GR_TILE;
    // All of a thread's loads before its first atomic (the atomics keep the program's order).
    unsigned long long k[GR_ITEMS];
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j) {
        const int64_t r = base + j * GR_THREADS + threadIdx.x;
        k[j] = r < n ? static_cast<unsigned long long>(__ldcs(keys + r)) : 0ull;
    }
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j)
        if (base + j * GR_THREADS + threadIdx.x < n) atomicAdd(&h[gr_region(k[j])], 1u);
    __syncthreads();
    if (threadIdx.x < GR_NB) counts[static_cast<int64_t>(threadIdx.x) * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(GR_THREADS) gr_partition_kernel(const long long *__restrict__ keys, int64_t n,
                                                                  int tiles, const unsigned *__restrict__ offs,
                                                                  unsigned long long *__restrict__ keys_p,
                                                                  unsigned *__restrict__ rows_p,
                                                                  unsigned short *__restrict__ loc) {
    __shared__ unsigned s_cnt[GR_NB], s_start[GR_NB + 1], s_goff[GR_NB];
    __shared__ unsigned long long s_key[GR_TILE];
    __shared__ unsigned short s_rel[GR_TILE];
    __shared__ unsigned char s_reg[GR_TILE];
    if (threadIdx.x < GR_NB) {
        s_cnt[threadIdx.x] = 0;
        s_goff[threadIdx.x] = offs[static_cast<int64_t>(threadIdx.x) * tiles + blockIdx.x];
    }
    __syncthreads();
    const int64_t base = static_cast<int64_t>(blockIdx.x) * GR_TILE;
    unsigned long long k[GR_ITEMS];
    unsigned rk[GR_ITEMS];
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j) {
        const int64_t r = base + j * GR_THREADS + threadIdx.x;
        k[j] = r < n ? static_cast<unsigned long long>(__ldcs(keys + r)) : 0ull;
    }
    // Slots within the tile's region runs, in any order: the ids do not depend on it.
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j)
        rk[j] = base + j * GR_THREADS + threadIdx.x < n ? atomicAdd(&s_cnt[gr_region(k[j])], 1u) : 0u;
    __syncthreads();
    if (threadIdx.x < 32) gr_starts([&](int b) { return s_cnt[b]; }, s_start);
    __syncthreads();
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j) {
        const int rel = j * GR_THREADS + threadIdx.x;
        if (base + rel >= n) continue;
        const unsigned b = gr_region(k[j]);
        const unsigned l = s_start[b] + rk[j];
        loc[base + rel] = static_cast<unsigned short>(l);
        s_key[l] = k[j];
        s_rel[l] = static_cast<unsigned short>(rel);
        s_reg[l] = static_cast<unsigned char>(b);
    }
    __syncthreads();
    const int rows = static_cast<int>(s_start[GR_NB]);
    for (int l = threadIdx.x; l < rows; l += GR_THREADS) {
        const unsigned b = s_reg[l];
        const unsigned p = s_goff[b] + static_cast<unsigned>(l) - s_start[b];
        keys_p[p] = s_key[l];
        rows_p[p] = static_cast<unsigned>(base) + s_rel[l];
    }
}

// One launch per step k of the regions' pipeline over three sub-tables: the inserts of region k
// (into table k % 3, cleared by the previous step), the smallest rows of region k - 1 (table
// (k - 1) % 3, whose inserts finished with the previous step) and the clearing of table
// (k + 1) % 3 (last read by the previous step) for region k + 1. Jobs with no rows are empty.
struct GrStep {
    unsigned ins0, ins1;  // positions of region k
    unsigned min0, min1;  // positions of region k - 1
    GroupTable ins, min, clr;
    int64_t clr_slots;  // 0: nothing to clear
};

__global__ void __launch_bounds__(256) gr_step_kernel(const unsigned long long *__restrict__ keys_p,
                                                      const unsigned *__restrict__ rows_p,
                                                      unsigned *__restrict__ slot_p, unsigned *__restrict__ min_p,
                                                      GrStep s, DevStatus *st) {
    const unsigned tid = blockIdx.x * blockDim.x + threadIdx.x;
    const unsigned p = s.ins0 + tid;
    if (p < s.ins1) {
        const unsigned long long key = keys_p[p];
        const unsigned row = rows_p[p];
        unsigned long long sl = 0;
        unsigned cur = 0xffffffffu;
        if (key != GI_EMPTY) {
            sl = gi_first(gmix(key), s.ins.mask);
            for (unsigned long long probes = 0;; ++probes) {
                unsigned long long va, vb;
                cas_pair(s.ins.words + 2 * sl, GI_EMPTY, ~0ull, key, 0xffffffff00000000ull | row, va, vb);
                if (va == GI_EMPTY) {
                    cur = row;
                    break;
                }
                if (va == key) {
                    cur = static_cast<unsigned>(vb);
                    break;
                }
                if (probes >= s.ins.mask) {
                    set_timeout(st);
                    break;
                }
                sl = gi_next(sl, s.ins.mask);
            }
        } else {
            cur = ld_relaxed32(&s.ins.meta(0)->x);
        }
        if (cur > row) atomicMin(&s.ins.meta(sl)->x, row);
        slot_p[p] = static_cast<unsigned>(sl);
    }
    const unsigned q = s.min0 + tid;
    if (q < s.min1) min_p[q] = s.min.meta(slot_p[q])->x;
    const int64_t stride = static_cast<int64_t>(gridDim.x) * blockDim.x;
    const ulonglong2 free_slot = make_ulonglong2(GI_EMPTY, ~0ull);
    for (int64_t i = tid; i < s.clr_slots; i += stride) reinterpret_cast<ulonglong2 *>(s.clr.words)[i] = free_slot;
}

// Row order again: each tile gathers its runs of min_p into shared memory in region-sorted
// order, then row i takes staged[loc[i]].
__global__ void __launch_bounds__(GR_THREADS) gr_restore_kernel(const unsigned *__restrict__ min_p,
                                                                const unsigned short *__restrict__ loc,
                                                                const unsigned *__restrict__ counts,
                                                                const unsigned *__restrict__ offs, int64_t n,
                                                                int tiles, unsigned *__restrict__ minrow) {
    __shared__ unsigned s_start[GR_NB + 1], s_goff[GR_NB];
    __shared__ unsigned s_vals[GR_TILE];
    if (threadIdx.x < 32) gr_starts([&](int b) { return counts[static_cast<int64_t>(b) * tiles + blockIdx.x]; }, s_start);
    if (threadIdx.x < GR_NB) s_goff[threadIdx.x] = offs[static_cast<int64_t>(threadIdx.x) * tiles + blockIdx.x];
    __syncthreads();
    const int rows = static_cast<int>(s_start[GR_NB]);
    unsigned at[GR_ITEMS];
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j) {
        const unsigned l = threadIdx.x + j * GR_THREADS;
        const int b = l < static_cast<unsigned>(rows) ? gr_region_of(s_start, l) : 0;
        at[j] = s_goff[b] + l - s_start[b];
    }
    unsigned v[GR_ITEMS];
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j) v[j] = threadIdx.x + j * GR_THREADS < rows ? __ldcs(min_p + at[j]) : 0u;
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j)
        if (threadIdx.x + j * GR_THREADS < rows) s_vals[threadIdx.x + j * GR_THREADS] = v[j];
    __syncthreads();
    const int64_t base = static_cast<int64_t>(blockIdx.x) * GR_TILE;
#pragma unroll
    for (int j = 0; j < GR_ITEMS; ++j) {
        const int64_t r = base + j * GR_THREADS + threadIdx.x;
        if (r < n) minrow[r] = s_vals[loc[r]];
    }
}

// The numbering of gi_number_kernel from each row's smallest row of its key: first occurrences
// (smallest row = the row) are ranked in row order by a decoupled lookback; a repeat takes the
// id of its first occurrence, from the tile's bitmap when that is in the same tile, else from
// the output row of the first occurrence (out starts as all ones; a bounded wait).
__global__ void __launch_bounds__(GI_THREADS, 4) gr_number_kernel(const unsigned *__restrict__ minrow, int64_t n,
                                                                  int tiles, unsigned long long *words, unsigned epoch,
                                                                  unsigned *counters, long long *out, DevStatus *st) {
    __shared__ unsigned long long s_prefix;
    __shared__ unsigned s_keep[GI_TILE / 32];
    __shared__ unsigned s_wpre[GI_TILE / 32];
    __shared__ long long s_out[GI_THREADS * GI_OUT_STRIDE];
    const int tile = take_ticket(counters);
    const int64_t t0 = static_cast<int64_t>(tile) * GI_TILE;
    const int64_t row0 = t0 + threadIdx.x * GI_ITEMS;
    unsigned mr[GI_ITEMS];
    if (row0 + GI_ITEMS <= n) {
        const uint4 *v = reinterpret_cast<const uint4 *>(minrow + row0);
#pragma unroll
        for (int q = 0; q < GI_ITEMS / 4; ++q) {
            const uint4 w = __ldcs(v + q);
            mr[4 * q] = w.x;
            mr[4 * q + 1] = w.y;
            mr[4 * q + 2] = w.z;
            mr[4 * q + 3] = w.w;
        }
    } else {
#pragma unroll
        for (int j = 0; j < GI_ITEMS; ++j) mr[j] = row0 + j < n ? minrow[row0 + j] : 0u;
    }
    int rel[GI_ITEMS];
    unsigned keep = 0;
#pragma unroll
    for (int j = 0; j < GI_ITEMS; ++j) {
        const int64_t r = row0 + j;
        rel[j] = -1;
        if (r < n) {
            rel[j] = static_cast<int>(static_cast<int64_t>(mr[j]) - t0);
            if (mr[j] == static_cast<unsigned>(r)) keep |= 1u << j;
        }
    }
    const unsigned odd = __shfl_down_sync(FULL, keep, 1);
    if (!(threadIdx.x & 1)) s_keep[threadIdx.x >> 1] = keep | (odd << 16);
    unsigned long long c = __popc(keep), tile_count;
    const unsigned long long off = block_exclusive_sum<unsigned long long>(c, &tile_count);
    if (!(threadIdx.x & 1)) s_wpre[threadIdx.x >> 1] = static_cast<unsigned>(off);
    if (threadIdx.x < 32) {
        unsigned long long pre = lookback_publish<4, CountRec>(words, tile, tile_count, 0ull, epoch, st);
        if (threadIdx.x == 0) s_prefix = pre;
    }
    __syncthreads();
    const unsigned prefix = static_cast<unsigned>(s_prefix);
#pragma unroll
    for (int j = 0; j < GI_ITEMS; ++j) {
        if (row0 + j >= n) continue;
        unsigned long long g;
        if (rel[j] >= 0) {
            const int w = rel[j] >> 5, bit = rel[j] & 31;
            g = prefix + s_wpre[w] + __popc(s_keep[w] & ((1u << bit) - 1u));
        } else {
            const unsigned long long *p = reinterpret_cast<const unsigned long long *>(out + mr[j]);
            unsigned it = 0;
            const unsigned limit = wait_limit(st);
            while ((g = ld_relaxed64(p)) == ~0ull) {
                if (++it > limit) {
                    set_timeout(st);
                    break;
                }
                backoff(it);
            }
        }
        s_out[threadIdx.x * GI_OUT_STRIDE + j] = static_cast<long long>(g);
    }
    __syncthreads();
    const int rows = static_cast<int>(n - t0 < GI_TILE ? n - t0 : GI_TILE);
    for (int i = threadIdx.x; i < rows; i += GI_THREADS)
        st_relaxed64(reinterpret_cast<unsigned long long *>(out + t0 + i),
                     static_cast<unsigned long long>(s_out[(i / GI_ITEMS) * GI_OUT_STRIDE + (i % GI_ITEMS)]));
    release_ticket(counters, tiles);
}

struct GroupScratch {
    vkc_array *words = nullptr;
    void release() {
        if (words) vkc_array_release(words);
        words = nullptr;
    }
};

// A table of `slots` slots (slot 0 included), every slot free.
static vkc_status new_table(vkc_ctx *ctx, uint64_t slots, bool pair, GroupScratch *g, GroupTable *t) {
    const int w = pair ? 4 : 2;
    const int64_t words = static_cast<int64_t>(w * slots);
    if (new_array(ctx, VKC_U64, words, false, &g->words)) return VKC_ALLOC;
    gi_clear_kernel<<<stream_grid(ctx, words / 2, 256, 8, 2048), 256, 0, ctx->stream>>>(
        static_cast<ulonglong2 *>(g->words->data()), words / 2, w);
    *t = GroupTable{static_cast<unsigned long long *>(g->words->data()), slots - 1, w};
    return launched(ctx, "gi_clear");
}

// One wave of resident blocks (the grid-stride loop gives every block the same share, so a
// second, partial wave would run at a fraction of the occupancy).
template <bool PAIR>
static void launch_insert(vkc_ctx *ctx, bool small, const long long *a, const long long *b, int64_t n,
                          const GroupTable &t, unsigned *slot_of, unsigned *flags) {
    static int resident[2] = {0, 0};
    auto kern = small ? gi_insert_kernel<PAIR, true> : gi_insert_kernel<PAIR, false>;
    int &per_sm = resident[small ? 1 : 0];
    if (per_sm == 0 && (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, GI_THREADS, 0) != cudaSuccess ||
                        per_sm < 1))
        per_sm = 1;
    const int grid = stream_grid(ctx, n, GI_THREADS, per_sm, GI_THREADS * GI_ROWS);
    kern<<<grid, GI_THREADS, 0, ctx->stream>>>(a, b, n, t, slot_of, flags, ctx->status);
}

int64_t scan_counts_sum_words(int64_t m);
void scan_counts(vkc_ctx *ctx, const unsigned *c, int64_t m, unsigned *sums, unsigned *out);

// Single keys, many distinct, at least GR_MIN_ROWS rows: the region-partitioned path above.
constexpr int64_t GR_MIN_ROWS = int64_t(1) << 22;

static vkc_status run_group_partitioned(vkc_ctx *ctx, const long long *keys, int64_t n, vkc_array *o) {
    const int tiles = static_cast<int>((n + GR_TILE - 1) / GR_TILE);
    const int64_t m = static_cast<int64_t>(GR_NB) * tiles;
    vkc_array *arr[10] = {};
    auto done = [&](vkc_status st) {
        for (vkc_array *a : arr)
            if (a) vkc_array_release(a);
        return st;
    };
    vkc_status st;
    const int64_t sizes[9] = {m, m, scan_counts_sum_words(m), n, n, (n + 1) / 2, n, n, n};
    const vkc_type types[9] = {VKC_I32, VKC_I32, VKC_I32, VKC_U64, VKC_I32, VKC_I32, VKC_I32, VKC_I32, VKC_I32};
    for (int i = 0; i < 9; ++i)
        if ((st = new_array(ctx, types[i], sizes[i], false, &arr[i]))) return done(st);
    auto *counts = static_cast<unsigned *>(arr[0]->data());
    auto *offs = static_cast<unsigned *>(arr[1]->data());
    auto *keys_p = static_cast<unsigned long long *>(arr[3]->data());
    auto *rows_p = static_cast<unsigned *>(arr[4]->data());
    auto *loc = static_cast<unsigned short *>(arr[5]->data());  // n u16 in (n + 1) / 2 words
    auto *slot_p = static_cast<unsigned *>(arr[6]->data());
    auto *min_p = static_cast<unsigned *>(arr[7]->data());
    auto *minrow = static_cast<unsigned *>(arr[8]->data());
    gr_count_kernel<<<tiles, GR_THREADS, 0, ctx->stream>>>(keys, n, tiles, counts);
    scan_counts(ctx, counts, m, static_cast<unsigned *>(arr[2]->data()), offs);
    gr_partition_kernel<<<tiles, GR_THREADS, 0, ctx->stream>>>(keys, n, tiles, offs, keys_p, rows_p, loc);
    if ((st = launched(ctx, "gr_partition"))) return done(st);
    // Region starts (offs of each region's first tile) on the host.
    void *h;
    if ((st = pinned(ctx, (GR_NB + 1) * sizeof(unsigned), &h))) return done(st);
    auto *starts = static_cast<unsigned *>(h);
    VKC_CUDA(ctx, cudaMemcpy2DAsync(starts, sizeof(unsigned), offs, static_cast<size_t>(tiles) * sizeof(unsigned),
                                    sizeof(unsigned), GR_NB, cudaMemcpyDeviceToHost, ctx->stream));
    VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
    std::vector<unsigned> start(starts, starts + GR_NB);
    start.push_back(static_cast<unsigned>(n));
    unsigned most = 1;
    for (int r = 0; r < GR_NB; ++r) most = std::max(most, start[r + 1] - start[r]);
    uint64_t slots = 2;
    while (slots < 2ull * most) slots <<= 1;
    if ((st = new_array(ctx, VKC_U64, static_cast<int64_t>(6 * slots), false, &arr[9]))) return done(st);
    auto *words = static_cast<unsigned long long *>(arr[9]->data());
    auto table = [&](int k) { return GroupTable{words + 2 * slots * static_cast<uint64_t>(k % 3), slots - 1, 2}; };
    gi_clear_kernel<<<stream_grid(ctx, static_cast<int64_t>(slots), 256, 8, 2048), 256, 0, ctx->stream>>>(
        reinterpret_cast<ulonglong2 *>(table(0).words), static_cast<int64_t>(slots), 2);
    for (int k = 0; k <= GR_NB; ++k) {
        GrStep s{};
        if (k < GR_NB) {
            s.ins0 = start[k];
            s.ins1 = start[k + 1];
        }
        if (k > 0) {
            s.min0 = start[k - 1];
            s.min1 = start[k];
        }
        s.ins = table(k);
        s.min = table(k + 2);  // (k - 1) % 3
        s.clr = table(k + 1);
        s.clr_slots = k + 1 < GR_NB ? static_cast<int64_t>(slots) : 0;
        const unsigned rows = std::max(s.ins1 - s.ins0, s.min1 - s.min0);
        const unsigned grid = std::max(1u, (rows + 255) / 256);
        gr_step_kernel<<<grid, 256, 0, ctx->stream>>>(keys_p, rows_p, slot_p, min_p, s, ctx->status);
    }
    if ((st = launched(ctx, "gr_regions"))) return done(st);
    gr_restore_kernel<<<tiles, GR_THREADS, 0, ctx->stream>>>(min_p, loc, counts, offs, n, tiles, minrow);
    VKC_CUDA(ctx, cudaMemsetAsync(o->data(), 0xff, static_cast<size_t>(n) * 8, ctx->stream));
    const int gtiles = static_cast<int>((n + GI_TILE - 1) / GI_TILE);
    unsigned long long *recs;
    if ((st = rec_arena(ctx, gtiles, &recs))) return done(st);
    gr_number_kernel<<<gtiles, GI_THREADS, 0, ctx->stream>>>(minrow, n, gtiles, recs, next_epoch(ctx), ctx->counters,
                                                            static_cast<long long *>(o->data()), ctx->status);
    return done(launched(ctx, "gr_number"));
}

static vkc_status run_group(vkc_ctx *ctx, const vkc_array *xa, const vkc_array *xb, vkc_value *out) {
    vkc_status st;
    int64_t n = xa->len;
    if (n >= (int64_t(1) << 31))
        return fail(ctx, VKC_USAGE, "group_id of " + std::to_string(n) + " rows: at most 2^31 - 1 rows per call");
    vkc_array *o;
    if ((st = new_array(ctx, VKC_I64, n, false, &o))) return st;
    if (n == 0) {
        out->kind = VKC_VALUE_ARRAY;
        out->array = o;
        return VKC_OK;
    }
    uint64_t slots = 2;
    while (slots < static_cast<uint64_t>(2 * n)) slots <<= 1;
    GroupScratch small, full;
    vkc_array *rows = nullptr, *flag_arr = nullptr;
    auto cleanup = [&]() {
        small.release();
        full.release();
        if (rows) vkc_array_release(rows);
        if (flag_arr) vkc_array_release(flag_arr);
    };
    auto alloc_fail = [&]() {
        cleanup();
        vkc_array_release(o);
        // group.rs:128-137 reports a failed table allocation.
        return fail(ctx, VKC_ALLOC, "cannot allocate a group_id table of " + std::to_string(slots) + " slots");
    };
    if (new_array(ctx, VKC_I32, n, false, &rows) || new_array(ctx, VKC_I32, 2, true, &flag_arr)) return alloc_fail();
    auto *slot_of = static_cast<unsigned *>(rows->data());
    auto *flags = static_cast<unsigned *>(flag_arr->data());
    const auto *a = static_cast<const long long *>(xa->data());
    const auto *b = xb ? static_cast<const long long *>(xb->data()) : nullptr;
    GroupTable t{};
    bool done = false;
    const uint64_t first_slots = uint64_t(1) << tune(ctx, TK_GROUP_FIRST_LOG2, n);
    if (slots > first_slots) {
        if ((st = new_table(ctx, first_slots, xb != nullptr, &small, &t))) {
            if (st == VKC_ALLOC) return alloc_fail();
            cleanup();
            vkc_array_release(o);
            return st;
        }
        if (xb) launch_insert<true>(ctx, true, a, b, n, t, slot_of, flags);
        else launch_insert<false>(ctx, true, a, b, n, t, slot_of, flags);
        if ((st = launched(ctx, "gi_insert"))) {
            cleanup();
            vkc_array_release(o);
            return st;
        }
        void *h;
        if ((st = pinned(ctx, 16, &h))) {
            cleanup();
            vkc_array_release(o);
            return st;
        }
        VKC_CUDA(ctx, cudaMemcpyAsync(h, flags, 8, cudaMemcpyDeviceToHost, ctx->stream));
        VKC_CUDA(ctx, cudaStreamSynchronize(ctx->stream));
        done = static_cast<unsigned *>(h)[1] == 0;
        if (!done) small.release();
        if (!done && !xb && n >= GR_MIN_ROWS) {
            // Many distinct single keys: the region-partitioned tables.
            st = run_group_partitioned(ctx, a, n, o);
            if (!st) {
                DevStatus ds;
                st = read_status(ctx, &ds);
            }
            cleanup();
            if (st) {
                vkc_array_release(o);
                return st;
            }
            out->kind = VKC_VALUE_ARRAY;
            out->array = o;
            return VKC_OK;
        }
    }
    if (!done) {
        if ((st = new_table(ctx, slots, xb != nullptr, &full, &t))) {
            if (st == VKC_ALLOC) return alloc_fail();
            cleanup();
            vkc_array_release(o);
            return st;
        }
        if (xb) launch_insert<true>(ctx, false, a, b, n, t, slot_of, flags);
        else launch_insert<false>(ctx, false, a, b, n, t, slot_of, flags);
        if ((st = launched(ctx, "gi_insert"))) {
            cleanup();
            vkc_array_release(o);
            return st;
        }
    }
    int tiles = static_cast<int>((n + GI_TILE - 1) / GI_TILE);
    unsigned long long *recs;
    if ((st = rec_arena(ctx, tiles, &recs))) {
        cleanup();
        vkc_array_release(o);
        return st;
    }
    gi_number_kernel<<<tiles, GI_THREADS, 0, ctx->stream>>>(slot_of, n, t, tiles, recs, next_epoch(ctx), ctx->counters,
                                                           static_cast<long long *>(o->data()), ctx->status);
    if ((st = launched(ctx, "gi_number"))) {
        cleanup();
        vkc_array_release(o);
        return st;
    }
    DevStatus ds;
    st = read_status(ctx, &ds);
    cleanup();
    if (st) {
        vkc_array_release(o);
        return st;
    }
    out->kind = VKC_VALUE_ARRAY;
    out->array = o;
    return VKC_OK;
}

// group.rs:260-277 (GroupId<i64>).
static vkc_status group_id_i64(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 1) return fail(ctx, VKC_RUNTIME, arity_error(1, nargs));
    if (!array_arg(ctx, args[0], VKC_I64, &st)) return st;
    return run_group(ctx, args[0].array, nullptr, out);
}

// group.rs:280-301 (GroupId2<i64, i64>).
static vkc_status group_id2_i64_i64(vkc_ctx *ctx, const vkc_value *args, int nargs, vkc_value *out) {
    vkc_status st;
    if (nargs != 2) return fail(ctx, VKC_RUNTIME, arity_error(2, nargs));
    if (!array_arg(ctx, args[0], VKC_I64, &st) || !array_arg(ctx, args[1], VKC_I64, &st)) return st;
    if (args[0].array->len != args[1].array->len)
        return fail(ctx, VKC_RUNTIME, "length mismatch: " + std::to_string(args[0].array->len) + " vs " +
                                          std::to_string(args[1].array->len));
    return run_group(ctx, args[0].array, args[1].array, out);
}

void register_group(std::vector<KernelDef> &t) {
    // group.rs:305-340: cost = key widths + 8.
    KernelDef d{"group_id_i64", VKC_WHOLE, {InSpec{IN_ARRAY, VKC_I64}}, true, VKC_I64, 16};
    d.whole = group_id_i64;
    t.push_back(d);
    d = KernelDef{"group_id2_i64_i64", VKC_WHOLE, {InSpec{IN_ARRAY, VKC_I64}, InSpec{IN_ARRAY, VKC_I64}}, true,
                  VKC_I64, 24};
    d.whole = group_id2_i64_i64;
    t.push_back(d);
}

}  // namespace vkc
