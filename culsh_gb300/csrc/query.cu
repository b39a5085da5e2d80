// K4: the query path.
//
// k_probe (one thread per (table, query)) replaces cuLSH_Kernels.cu:266-289
// (kernel_calculateDeltas), cuLSH_Kernels.cu:144-257 (balanceHeap_deltas +
// kernel_calculateProbingCodes), cuLSH_Querying.cu:63-119 (the host round trip
// that scatters home codes) and the whole sort-merge bucket match of
// cuLSH_Querying.cu:124-165 + cuLSH_Kernels.cu:124-138: every probe code is
// packed into the table's key layout and looked up in the open-addressing hash
// built at index time, verified against the stored bucket key. It also sums
// the non-unique candidate counts of cuLSH_SearchTables.cu:250-255.
//
// k_candidates (one 128-thread block per query) replaces the host collect /
// sort / unique of cuLSH_SearchTables.cu:321-364, the per-query fill_n of
// :384-389, kernel_calculateDistances (cuLSH_Kernels.cu:301-348) and the top-K
// kernels (cuLSH_Kernels.cu:356-456): bucket ids are gathered straight from the
// sorted id arrays, deduplicated in a shared-memory hash set (global arena for
// large sets), squared L2 distances are computed in the reference's lane order
// from 16-byte loads, and each warp keeps a sorted top-K that the block merges.
#include <atomic>
#include <cfloat>
#include <cstdlib>
#include <utility>

#include "culsh_internal.cuh"
#include "topk_common.cuh"

namespace culsh {
namespace {

constexpr int CT = 128;
constexpr int CW = CT / 32;
constexpr int SM_SLOTS = 4096;
constexpr int SM_CAP = SM_SLOTS / 2;
constexpr int GCH = 256;   // bucket slots scanned per gather chunk

__device__ __forceinline__ int ceil_log2_dev(int n) {
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

// Max-heap sift-down over delta indices; an empty slot (-1) ranks above every
// delta (cuLSH_Kernels.cu:144-175).
__device__ void sift_deltas(int8_t* perm, const float* dl, int total, int levels) {
    int parent = 0;
    for (int level = 0; level < levels - 1; ++level) {
        const int left = parent * 2 + 1, right = left + 1;
        int mx = parent;
        if (left < total && perm[left] == -1) {
            mx = left;
        } else if (right < total && perm[right] == -1) {
            mx = right;
        } else {
            if (left < total && dl[perm[left]] > dl[perm[mx]]) mx = left;
            if (right < total && dl[perm[right]] > dl[perm[mx]]) mx = right;
        }
        if (mx == parent) break;
        const int8_t t = perm[parent];
        perm[parent] = perm[mx];
        perm[mx] = t;
        parent = mx;
    }
}

// Exact-code lookup of one probe row in table l; returns the bucket index
// within the table or -1.
__device__ int32_t lookup_row(const LookupView& lv, int l, const float* row) {
    uint32_t key[kMaxKW];
#pragma unroll
    for (int w = 0; w < kMaxKW; ++w) key[w] = 0;
    const int M = lv.M, KW = lv.KW;
    uint64_t hs = 0;
    for (int m = 0; m < M; ++m) {
        const int c = l * M + m;
        const float f = row[m];
        if (!(f >= -2147483648.0f && f < 2147483648.0f)) return -1;
        const int32_t ci = (int32_t)f;
        const int32_t lo = __ldg(lv.cmin + c);
        if (ci < lo || ci > __ldg(lv.cmax + c)) return -1;
        const int bits = __ldg(lv.fbits + c);
        if (bits) key_put(key, __ldg(lv.foff + c), bits, (uint32_t)(ci - lo));
        hs += (uint64_t)(uint32_t)(ci - lo) * __ldg(lv.rmul + c);
    }
    const uint32_t gmask = __ldg(lv.hmask + l);
    const uint64_t hh = hash_finish(hs);
    const uint32_t h = (uint32_t)hh;
    const uint32_t fp = slot_fp(hh);
    const unsigned long long* slots = lv.hslots + __ldg(lv.hoff + l);
    const uint64_t bo = __ldg(lv.boff + l);
    for (uint32_t p = 0; p <= gmask; ++p) {
        const unsigned long long* grp = slots + (uint64_t)((h + p) & gmask) * kGroupWords;
        const unsigned long long fps = __ldg(grp);
        for (int g = 0; g < kGroupSlots; ++g) {
            const uint32_t f = (uint32_t)(fps >> (16 * g)) & 0xFFFFu;
            if (f == kEmptyFp) return -1;
            if (f == fp) {
                const uint32_t j = __ldg(reinterpret_cast<const uint32_t*>(grp + 1) + g);
                const uint32_t* uk = lv.ukeys + (bo + j) * KW;
                bool eq = true;
                for (int w = 0; w < KW; ++w) eq &= __ldg(uk + w) == key[w];
                if (eq) return (int32_t)j;
            }
        }
    }
    return -1;
}

__global__ void __launch_bounds__(128) k_probe(ProbeArgs a) {
    const LookupView& lv = a.lv;
    const int Q = a.Q, T = a.T, L = lv.L, M = lv.M;
    const int64_t idx = (int64_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (idx >= (int64_t)L * Q) return;
    const int l = (int)(idx / Q), q = (int)(idx - (int64_t)l * Q);

    float home[kMaxM], row[kMaxM], dl[2 * kMaxM];
    for (int m = 0; m < M; ++m) {
        const float v = a.vals[(int64_t)(l * M + m) * Q + q];
        const float f = floorf(v);
        const float down = __fsub_rn(v, f);
        home[m] = f;
        dl[m] = down;
        dl[m + M] = __fsub_rn(1.0f, down);
    }
    int32_t* qb = a.qbuckets + (int64_t)l * Q * T + (int64_t)q * T;
    const uint64_t bo = lv.boff[l];
    unsigned long long cnu = 0;
    {
        const int32_t j = lookup_row(lv, l, home);
        qb[0] = j;
        if (j >= 0) cnu += lv.sizes[bo + j];
    }
    if (T > 1) {
        // Heap selection of the (at most 64) smallest deltas, then heap sort
        // into ascending order (cuLSH_Kernels.cu:202-214).
        const int maxT = min(2 * M, 64);
        const int levels = ceil_log2_dev(2 * M + 1);
        int8_t perm[64];
        for (int i = 0; i < maxT; ++i) perm[i] = -1;
        for (int i = 0; i < 2 * M; ++i) {
            if (perm[0] == -1 || dl[i] < dl[perm[0]]) {
                perm[0] = (int8_t)i;
                sift_deltas(perm, dl, maxT, levels);
            }
        }
        for (int i = maxT - 1; i > 0; --i) {
            const int8_t t = perm[0];
            perm[0] = perm[i];
            perm[i] = t;
            sift_deltas(perm, dl, i, levels);
        }
        // Shift / expand enumeration with a linear minimum search
        // (cuLSH_Kernels.cu:216-255); 64-bit masks.
        uint64_t comb[kMaxT];
        float cd[kMaxT];
        comb[0] = 1;
        cd[0] = dl[perm[0]];
        int size = 1;
        for (int t = 1; t < T; ++t) {
            float mn = FLT_MAX;
            int mi = 0;
            for (int i = 0; i < size; ++i) {
                if (cd[i] < mn) {
                    mi = i;
                    mn = cd[i];
                }
            }
            uint64_t probe = comb[mi];
            for (int m = 0; m < M; ++m) row[m] = home[m];
            int top = 0;
            for (uint64_t bitsleft = probe; bitsleft; bitsleft &= bitsleft - 1) {
                const int i = __ffsll((long long)bitsleft) - 1;
                const int pi = perm[i];
                const int m = pi % M;
                row[m] = __fadd_rn(row[m], pi >= M ? 1.0f : -1.0f);
                top = i;
            }
            if (top < maxT - 1) {
                probe |= 1ull << (top + 1);
                mn = __fadd_rn(mn, dl[perm[top + 1]]);
                comb[mi] = probe;
                cd[mi] = mn;
                probe -= 1ull << top;
                mn = __fsub_rn(mn, dl[perm[top]]);
                comb[size] = probe;
                cd[size] = mn;
                ++size;
            }
            const int32_t j = lookup_row(lv, l, row);
            qb[t] = j;
            if (j >= 0) cnu += lv.sizes[bo + j];
        }
    }
    if (cnu) atomicAdd(a.cnu + q, cnu);
}


// ---------------------------------------------------------------------------
// Fast multiprobe path for the common shapes: M <= 32 columns, T <= 64
// probes, packed keys of at most 128 bits and codes below 2^24 in magnitude
// (so that the reference's float +-1 on a code equals integer +-1).
//
// The reference orders the 2M deltas with a heap sort (cuLSH_Kernels.cu:202-214).
// When the deltas are pairwise distinct every correct sort yields that same
// order, so the kernel ranks the M "down" deltas and takes the "up" deltas
// (1 - down, a non-increasing function of down) in reverse, then merges the
// two lists; any tie or NaN sends the thread through the reference's heap
// procedure instead. The shift/expand enumeration then runs exactly as in
// k_probe. A probe's key is the home key plus or minus one unit of each
// perturbed column's field (packing is linear) in 128-bit modular arithmetic,
// and column range validity is three bit masks. Group loads are issued four
// at a time before any is consumed. Per-thread state lives in a strided
// slice of shared memory. Results equal k_probe's exactly.
constexpr int PF = 128;
typedef unsigned __int128 u128;

__device__ __forceinline__ u128 field_term(int64_t f, int off) { return ((u128)(__int128)f) << off; }

__device__ __forceinline__ int lowest_bit(uint32_t b) { return __ffs((int)b) - 1; }
__device__ __forceinline__ int lowest_bit(uint64_t b) { return __ffsll((long long)b) - 1; }
__device__ __forceinline__ int highest_bit(uint32_t b) { return 31 - __clz((int)b); }
__device__ __forceinline__ int highest_bit(uint64_t b) { return 63 - __clzll((long long)b); }

struct FastProbeCtx {
    u128 hkey;
    uint64_t h0;                        // additive lookup hash of the home key (before the mix)
    uint32_t ok0, okUp, okDn, allM;     // per-column range validity (M <= 32)
    const uint8_t* enc;                 // sorted delta i -> column | (up << 7); strided slice
    const unsigned long long* funit;    // this table's field units 2^foff (low, high)
    const unsigned long long* rmul;     // this table's hash multipliers
};

__device__ __forceinline__ u128 unit_of(const unsigned long long* funit, int m) {
    return ((u128)__ldg(funit + 2 * m + 1) << 64) | (u128)__ldg(funit + 2 * m);
}

// Key of a probe mask; returns false when a column leaves [cmin, cmax]. A
// column perturbed both up and down keeps its home code.
template <typename MaskT>
__device__ __forceinline__ bool probe_key(const FastProbeCtx& c, MaskT mask, u128& key) {
    uint32_t up = 0, dn = 0;
    for (MaskT b = mask; b; b &= b - 1) {
        const int e = c.enc[lowest_bit(b) * PF];
        if (e & 0x80) up |= 1u << (e & 0x3f);
        else dn |= 1u << (e & 0x3f);
    }
    const uint32_t nu = up & ~dn, nd = dn & ~up;
    if ((~(nu | nd) & c.allM & ~c.ok0) | (nu & ~c.okUp) | (nd & ~c.okDn)) return false;
    u128 k = c.hkey;
    for (uint32_t b = nu; b; b &= b - 1) k += unit_of(c.funit, lowest_bit(b));
    for (uint32_t b = nd; b; b &= b - 1) k -= unit_of(c.funit, lowest_bit(b));
    key = k;
    return true;
}

// Lookup hash of a probe mask (the home hash +- the multiplier of every
// perturbed column, accumulated in the same walk over the mask: a column
// perturbed both up and down adds +R - R = 0 mod 2^64, as it keeps its home
// code); returns false when a column leaves [cmin, cmax].
template <typename MaskT>
__device__ __forceinline__ bool probe_hash(const FastProbeCtx& c, MaskT mask, uint64_t& hh) {
    uint32_t up = 0, dn = 0;
    uint64_t h = c.h0;
    for (MaskT b = mask; b; b &= b - 1) {
        const int e = c.enc[lowest_bit(b) * PF];
        const uint64_t r = __ldg(c.rmul + (e & 0x3f));
        if (e & 0x80) {
            up |= 1u << (e & 0x3f);
            h += r;
        } else {
            dn |= 1u << (e & 0x3f);
            h -= r;
        }
    }
    const uint32_t nu = up & ~dn, nd = dn & ~up;
    if ((~(nu | nd) & c.allM & ~c.ok0) | (nu & ~c.okUp) | (nd & ~c.okDn)) return false;
    hh = hash_finish(h);
    return true;
}

__device__ __forceinline__ bool key_matches(const uint32_t* uk, u128 k, int KW) {
    bool eq = __ldg(uk) == (uint32_t)k;
    if (KW > 1) eq &= __ldg(uk + 1) == (uint32_t)(k >> 32);
    if (KW > 2) eq &= __ldg(uk + 2) == (uint32_t)(k >> 64);
    if (KW > 3) eq &= __ldg(uk + 3) == (uint32_t)(k >> 96);
    return eq;
}

// The reference's heap selection + heap sort over a strided slice (used
// only when deltas tie or are NaN). val(i) is delta i; perm[] receives the
// delta indices in ascending order.
template <class V>
__device__ void heap_order_strided(V val, int8_t* perm, int M2, int maxT) {
    const int levels = ceil_log2_dev(M2 + 1);
    auto sift = [&](int total) {
        int parent = 0;
        for (int level = 0; level < levels - 1; ++level) {
            const int left = parent * 2 + 1, right = left + 1;
            int mx = parent;
            const int pl = left < total ? perm[left * PF] : 0, pr = right < total ? perm[right * PF] : 0;
            if (left < total && pl == -1) {
                mx = left;
            } else if (right < total && pr == -1) {
                mx = right;
            } else {
                float best = val(perm[parent * PF]);
                if (left < total && val(pl) > best) {
                    mx = left;
                    best = val(pl);
                }
                if (right < total && val(pr) > best) mx = right;
            }
            if (mx == parent) break;
            const int8_t t = perm[parent * PF];
            perm[parent * PF] = perm[mx * PF];
            perm[mx * PF] = t;
            parent = mx;
        }
    };
    for (int i = 0; i < maxT; ++i) perm[i * PF] = -1;
    for (int i = 0; i < M2; ++i) {
        const int p0 = perm[0];
        if (p0 == -1 || val(i) < val(p0)) {
            perm[0] = (int8_t)i;
            sift(maxT);
        }
    }
    for (int i = maxT - 1; i > 0; --i) {
        const int8_t t = perm[0];
        perm[0] = perm[i * PF];
        perm[i * PF] = t;
        sift(i);
    }
}

// Batcher's odd-even merge-sort network for N keys (any N), built at compile
// time: comparator i orders keys a[i] < b[i]. N = 8, 12, 16 give 19, 42, 63
// comparators.
template <int N>
struct SortNet {
    int a[64], b[64], n;
    constexpr SortNet() : a{}, b{}, n(0) {
        for (int p = 1; p < N; p <<= 1)
            for (int k = p; k >= 1; k >>= 1)
                for (int j = k % p; j + k < N; j += 2 * k)
                    for (int i = 0; i < k && i < N - j - k; ++i)
                        if ((i + j) / (2 * p) == (i + j + k) / (2 * p)) {
                            a[n] = i + j;
                            b[n] = i + j + k;
                            ++n;
                        }
    }
};
template <int N>
constexpr SortNet<N> kSortNet{};

template <int A, int B, int N>
__device__ __forceinline__ void compare_swap(float (&v)[N], uint32_t (&pl)[N]) {
    const bool sw = v[B] < v[A];
    const float lo = sw ? v[B] : v[A], hi = sw ? v[A] : v[B];
    const uint32_t plo = sw ? pl[B] : pl[A], phi = sw ? pl[A] : pl[B];
    v[A] = lo;
    v[B] = hi;
    pl[A] = plo;
    pl[B] = phi;
}

template <int N, size_t... I>
__device__ __forceinline__ void sort_network(float (&v)[N], uint32_t (&pl)[N], std::index_sequence<I...>) {
    (compare_swap<kSortNet<N>.a[I], kSortNet<N>.b[I]>(v, pl), ...);
}

// Orders the 2M deltas of one (table, query) pair in registers for M <= MM:
// the downs are sorted by a network (payload: column), each down's place in
// the merged sequence is its rank plus the number of ups below it, and the
// ups fill the remaining places in ascending order (ups fall as downs rise).
// Writes enc[] (sorted delta -> column | up << 7) and returns whether all 2M
// values are distinct and strictly ascending; otherwise the caller takes the
// reference's heap procedure.
template <int MM, class SV>
__device__ __forceinline__ bool order_deltas_net(const float* dn, uint8_t* enc, int M, SV sv) {
    float v[MM];
    uint32_t col[MM];
#pragma unroll
    for (int k = 0; k < MM; ++k) {
        v[k] = k < M ? dn[k * PF] : 2.0f;   // padding sorts last
        col[k] = (uint32_t)k;
    }
    sort_network<MM>(v, col, std::make_index_sequence<kSortNet<MM>.n>{});
    float u[MM];
#pragma unroll
    for (int k = 0; k < MM; ++k) u[k] = __fsub_rn(1.0f, v[k]);   // padding: -1, below every value
    uint32_t taken = 0;
#pragma unroll
    for (int k = 0; k < MM; ++k) {
        if (k < M) {
            int below = 0;
#pragma unroll
            for (int k2 = 0; k2 < MM; ++k2) below += u[k2] < v[k];
            const int pos = k + below - (MM - M);
            taken |= 1u << pos;
            enc[pos * PF] = (uint8_t)col[k];
        }
    }
#pragma unroll
    for (int k = MM - 1; k >= 0; --k) {
        if (k < M) {
            const int pos = __ffs((int)~taken) - 1;
            taken |= 1u << pos;
            enc[pos * PF] = (uint8_t)(col[k] | 0x80u);
        }
    }
    bool ok = true;
    float prev = sv(0);
#pragma unroll
    for (int o = 1; o < 2 * MM; ++o) {
        if (o < 2 * M) {
            const float x = sv(o);
            ok &= prev < x;
            prev = x;
        }
    }
    return ok;
}

// The reference's heap procedure over a pair's 2M deltas, for the rare pairs
// whose deltas tie (or are NaN). Out of line: inlined, its loops enlarge the
// probe kernel and slow every pair. dn: the pair's downs (strided slice);
// enc: receives sorted delta -> column | up << 7.
__device__ __noinline__ void order_deltas_heap(const float* dn, uint8_t* enc, int M) {
    auto dv = [&](int i) {
        const float d = dn[(i < M ? i : i - M) * PF];
        return i < M ? d : __fsub_rn(1.0f, d);
    };
    const int M2 = 2 * M;
    int8_t* perm = reinterpret_cast<int8_t*>(enc);
    heap_order_strided(dv, perm, M2, M2);
    for (int i = 0; i < M2; ++i) {
        const int pm = perm[i * PF];
        enc[i * PF] = (uint8_t)((pm % M) | (pm >= M ? 0x80 : 0));
    }
}

// Entries kept in the enumeration's candidate list. Picked sums never
// decrease (an expansion adds a delta, a shift trades a delta for a later,
// larger one), so a candidate with r candidates before it in pick order
// (sum, then insertion order) is picked r + 1 steps later at the earliest;
// once the list holds more than ceil(T/2) + 1, its last one can no longer be
// among the remaining picks and is dropped (the others keep their order, so
// ties still go to the earlier candidate). Only for T > 16, where the list
// sets the shared memory per thread and hence the occupancy.
__host__ __device__ constexpr int probe_cand_cap(int T) { return T > 16 ? (T + 1) / 2 + 1 : T; }
// Slots of the list: one more than the cap while capping, for the entry
// appended before the drop; T - 1 otherwise (step t < T - 1 appends at most
// at index t; the last step, T - 1, does not expand: nothing reads the list
// after it).
__host__ __device__ constexpr int probe_cand_slots(int T) {
    return T > 16 ? probe_cand_cap(T) + 1 : (T > 1 ? T - 1 : 1);
}

// Per-thread shared-memory slice of the fast kernel, in bytes per thread;
// the rank slice ord[M] only where the deltas are ordered in shared memory.
template <typename MaskT>
__host__ __device__ constexpr size_t probe_fast_bytes_per_thread(int M, int T, bool ranks = true) {
    return sizeof(MaskT) * (size_t)probe_cand_slots(T) + sizeof(float) * (size_t)(M + probe_cand_slots(T)) +
           (size_t)(2 * M + (ranks ? M : 0));
}

// PCH: probes whose group loads are in flight together (tuned: 1, 2 or 4).
// MM > 0: M <= MM, deltas ordered in registers (order_deltas_net); MM = 0:
// ranking and merge over the shared-memory slice.
// kForm: 0 fused (enumeration with batched lookups), 1 split (enumeration
// only; k_probe_resolve looks up), 2 tail (enumerate every probe, then look
// them all up behind the key filter at the end of the same kernel).
template <typename MaskT, int PCH, int MM, int kForm>
__global__ void __launch_bounds__(PF, kForm == 2 && MM <= 12 ? 9 : (kForm > 0 ? 8 : 6)) k_probe_fast(ProbeArgs a) {
    extern __shared__ __align__(16) unsigned char psm[];
    const LookupView& lv = a.lv;
    const int Q = a.Q, T = a.T, L = lv.L, M = lv.M, KW = lv.KW;
    const int tid = threadIdx.x;
    const int M2 = 2 * M;
    // Strided per-thread slices (element i of a thread at [i * PF + tid]):
    // comb[S] (MaskT), dn[M], cd[S] (f32), enc[2M] (sorted delta -> column
    // | up << 7), ord[M] (u8; MM = 0 only), S = probe_cand_slots(T). Each slice is placed
    // from the block's base; the thread offset is added last, in units of the
    // slice's own element type.
    const int CAP = probe_cand_cap(T), SLOTS = probe_cand_slots(T);
    size_t off = 0;
    MaskT* comb = reinterpret_cast<MaskT*>(psm + off) + tid;
    off += sizeof(MaskT) * (size_t)SLOTS * PF;
    float* dn = reinterpret_cast<float*>(psm + off) + tid;
    float* cd = reinterpret_cast<float*>(psm + off) + M * PF + tid;
    off += sizeof(float) * (size_t)(M + SLOTS) * PF;
    uint8_t* enc = psm + off + tid;
    uint8_t* ord = psm + off + M2 * PF + tid;
    // value of delta i (i < M: down of column i; else up of column i - M,
    // 1 - down as the reference computes it)
    auto dv = [&](int i) {
        const float d = dn[(i < M ? i : i - M) * PF];
        return i < M ? d : __fsub_rn(1.0f, d);
    };
    // value of sorted delta i
    auto sv = [&](int i) {
        const int e = enc[i * PF];
        const float d = dn[(e & 0x3f) * PF];
        return (e & 0x80) ? __fsub_rn(1.0f, d) : d;
    };
    const int64_t idx = (int64_t)blockIdx.x * PF + tid;
    if (idx >= (int64_t)L * Q) return;   // no block-level synchronisation below
    const int l = (int)(idx / Q), q = (int)(idx - (int64_t)l * Q);

    FastProbeCtx c;
    c.hkey = 0;
    c.ok0 = c.okUp = c.okDn = 0;
    c.allM = M >= 32 ? ~0u : ((1u << M) - 1);
    c.enc = enc;
    c.funit = lv.funit + 2 * l * M;
    c.rmul = lv.rmul + l * M;
    c.h0 = 0;
    bool distinct = true;
    for (int m = 0; m < M; ++m) {
        const int col = l * M + m;
        const float v = a.vals[(int64_t)col * Q + q];
        const float f = floorf(v);
        const float down = __fsub_rn(v, f);
        const float up = __fsub_rn(1.0f, down);
        dn[m * PF] = down;
        distinct &= (down == down) && (up == up);
        const int64_t lo = __ldg(lv.cmin + col), hi = __ldg(lv.cmax + col);
        const int64_t h = (f >= -1.0e15f && f <= 1.0e15f) ? (int64_t)f : (int64_t)1 << 50;
        c.ok0 |= (uint32_t)(h >= lo && h <= hi) << m;
        c.okUp |= (uint32_t)(h + 1 >= lo && h + 1 <= hi) << m;
        c.okDn |= (uint32_t)(h - 1 >= lo && h - 1 <= hi) << m;
        c.hkey += field_term(h - lo, __ldg(lv.foff + col));
        c.h0 += (uint64_t)(h - lo) * __ldg(c.rmul + m);
    }

    if (T > 1 && MM > 0) {
        if (distinct) distinct = order_deltas_net<(MM > 0 ? MM : 1)>(dn, enc, M, sv);
        if (!distinct) order_deltas_heap(dn, enc, M);
        comb[0] = 1;
        cd[0] = sv(0);
    } else if (T > 1) {
        // Rank the downs (ties or NaN fall back to the heap procedure).
        for (int i = 0; i < M && distinct; ++i) {
            const float di = dn[i * PF];
            int r = 0;
            for (int j = 0; j < M; ++j) {
                const float dj = dn[j * PF];
                r += dj < di;
                distinct &= (j == i) | (dj != di);
            }
            ord[r * PF] = (uint8_t)i;
        }
        // Ups in reverse down order must be strictly increasing, then merge.
        if (distinct) {
            for (int k = 1; k < M && distinct; ++k)
                distinct &= dv(ord[(M - k) * PF] + M) < dv(ord[(M - 1 - k) * PF] + M);
        }
        if (distinct) {
            int id = 0, iu = M - 1;
            for (int o = 0; o < M2; ++o) {
                const float vd = id < M ? dn[ord[id * PF] * PF] : FLT_MAX;
                const float vu = iu >= 0 ? dv(ord[iu * PF] + M) : FLT_MAX;
                const bool take_down = iu < 0 || (id < M && vd < vu);
                if (id < M && iu >= 0 && vd == vu) {
                    distinct = false;
                    break;
                }
                const int m = take_down ? ord[id * PF] : ord[iu * PF];
                enc[o * PF] = (uint8_t)(m | (take_down ? 0 : 0x80));
                if (take_down) ++id;
                else --iu;
            }
        }
        if (!distinct) order_deltas_heap(dn, enc, M);
        comb[0] = 1;
        cd[0] = sv(0);
    }

    int32_t* qb = a.qbuckets + (int64_t)l * Q * T + (int64_t)q * T;
    int size = 1;
    // One enumeration step (cuLSH_Kernels.cu:216-255): probe t > 0 is the
    // candidate of smallest delta sum (the first of equal sums), which is
    // then shifted in place and expanded into a new candidate.
    auto next_probe = [&](bool expand) -> MaskT {
        float mn = FLT_MAX;
        int mi = 0;
        for (int i = 0; i < size; ++i) {
            const float x = cd[i * PF];
            if (x < mn) {
                mi = i;
                mn = x;
            }
        }
        const MaskT probe = comb[mi * PF];
        const int top = highest_bit(probe);
        if (expand && top < M2 - 1) {
            const MaskT p1 = probe | ((MaskT)1 << (top + 1));
            const float m1 = __fadd_rn(mn, sv(top + 1));
            comb[mi * PF] = p1;
            cd[mi * PF] = m1;
            comb[size * PF] = p1 - ((MaskT)1 << top);
            cd[size * PF] = __fsub_rn(m1, sv(top));
            ++size;
            if (size > CAP) {   // drop the last candidate in pick order (see probe_cand_cap)
                float mx = -FLT_MAX;
                int mj = 0;
                for (int i = 0; i < size; ++i) {
                    const float x = cd[i * PF];
                    if (x >= mx) {
                        mx = x;
                        mj = i;
                    }
                }
                for (int i = mj; i + 1 < size; ++i) {
                    comb[i * PF] = comb[(i + 1) * PF];
                    cd[i * PF] = cd[(i + 1) * PF];
                }
                --size;
            }
        }
        return probe;
    };
    if constexpr (kForm > 0) {
        if constexpr (kForm == 1) {
            // Pair context for the lookup kernel: home key and sorted deltas.
            uint32_t ew[8];
#pragma unroll
            for (int w = 0; w < 8; ++w) ew[w] = 0;
            if (T > 1) {
#pragma unroll
                for (int i = 0; i < 32; ++i)
                    if (i < M2) ew[i >> 2] |= (uint32_t)enc[i * PF] << (8 * (i & 3));
            }
            uint4* cx = a.pctx + idx * 3;
            cx[0] = make_uint4((uint32_t)c.hkey, (uint32_t)(c.hkey >> 32), (uint32_t)(c.hkey >> 64),
                               (uint32_t)(c.hkey >> 96));
            cx[1] = make_uint4(ew[0], ew[1], ew[2], ew[3]);
            cx[2] = make_uint4(ew[4], ew[5], ew[6], ew[7]);
        }
        // Hash and mask of probe t at [l][t][q] (a warp's stores coalesce);
        // split form: the query buckets are staged four at a time for
        // 16-byte stores; tail form: the probe's filter word is prefetched
        // into L2 for the lookups at the end.
        const int64_t base = (int64_t)l * T * Q + q;
        const bool vec = (T & 3) == 0;
        const uint32_t* filt = lv.filt ? lv.filt + __ldg(lv.fl_off + l) : nullptr;
        const uint32_t fmask = lv.filt ? __ldg(lv.fl_mask + l) : 0u;
        // Tail form: the filter word of probe t is loaded as the probe is
        // made and checked one probe later (the next enumeration step hides
        // its latency); `pass` collects the probes the filter lets through.
        uint64_t pass = 0;
        uint32_t pfw = 0u, pneed = 1u;
        int pt = -1;
        int s0 = -1, s1 = -1, s2 = -1, s3 = -1;
        for (int t = 0; t < T; ++t) {
            const MaskT probe = t > 0 ? next_probe(t < T - 1) : (MaskT)0;
            uint64_t hh;
            const bool ok = probe_hash(c, probe, hh);
            if (ok) {
                a.ph[base + (int64_t)t * Q] = hh;
                a.pmask[base + (int64_t)t * Q] = (uint32_t)probe;
            }
            if constexpr (kForm == 2) {
                if (pt >= 0 && (pfw & pneed) == pneed) pass |= 1ull << pt;
                pt = -1;
                if (ok) {
                    const uint32_t fx = filter_mix(hh);
                    pneed = filter_bits(fx);
                    pfw = filt ? __ldg(filt + (fx & fmask)) : ~0u;
                    pt = t;
                }
            }
            if constexpr (kForm == 1) {
                const int v = ok ? -2 : -1;
                if (vec) {
                    const int r = t & 3;
                    s0 = r == 0 ? v : s0;
                    s1 = r == 1 ? v : s1;
                    s2 = r == 2 ? v : s2;
                    s3 = r == 3 ? v : s3;
                    if (r == 3) *reinterpret_cast<int4*>(qb + t - 3) = make_int4(s0, s1, s2, s3);
                } else {
                    qb[t] = v;
                }
            }
        }
        if constexpr (kForm == 2) {
            if (pt >= 0 && (pfw & pneed) == pneed) pass |= 1ull << pt;
            // Every probe a miss, then the few the filter passed: walk the
            // hash group, verify the key (the pair's context is still here).
            for (int t4 = 0; t4 < T; t4 += 4) {
                if (vec) {
                    *reinterpret_cast<int4*>(qb + t4) = make_int4(-1, -1, -1, -1);
                } else {
                    for (int k = t4; k < t4 + 4 && k < T; ++k) qb[k] = -1;
                }
            }
            const uint32_t gmask = __ldg(lv.hmask + l);
            const unsigned long long* slots = lv.hslots + __ldg(lv.hoff + l);
            const uint64_t bo = __ldg(lv.boff + l);
            unsigned long long cnu = 0;
#pragma unroll 1
            for (; pass; pass &= pass - 1) {
                const int t = __ffsll((long long)pass) - 1;
                const uint64_t hh = a.ph[base + (int64_t)t * Q];
                const MaskT pm = (MaskT)a.pmask[base + (int64_t)t * Q];
                const uint32_t fp = slot_fp(hh);
                uint32_t h = (uint32_t)hh & gmask;
                int32_t res = -1;
                bool done = false;
                for (uint32_t p = 0; p <= gmask && !done; ++p) {
                    const unsigned long long* grp = slots + (uint64_t)h * kGroupWords;
                    const unsigned long long w = __ldg(grp);
                    for (int e = 0; e < kGroupSlots && !done; ++e) {
                        const uint32_t f = (uint32_t)(w >> (16 * e)) & 0xFFFFu;
                        if (f == kEmptyFp) {
                            done = true;
                        } else if (f == fp) {
                            const uint32_t bj = __ldg(reinterpret_cast<const uint32_t*>(grp + 1) + e);
                            u128 k;
                            probe_key(c, pm, k);
                            if (key_matches(lv.ukeys + (bo + bj) * KW, k, KW)) {
                                res = (int32_t)bj;
                                done = true;
                            }
                        }
                    }
                    h = (h + 1) & gmask;
                }
                if (res >= 0) {
                    qb[t] = res;
                    cnu += __ldg(lv.sizes + bo + res);
                }
            }
            if (cnu) atomicAdd(a.cnu + q, cnu);
        }
        return;
    }

    // Probes: enumerate PCH at a time, issue the group loads of the batch
    // together, then resolve each probe: walk its group's fingerprints
    // (registers) until an empty slot, verifying the stored key on a
    // fingerprint match.
    const uint32_t gmask = __ldg(lv.hmask + l);
    const unsigned long long* slots = lv.hslots + __ldg(lv.hoff + l);
    const uint64_t bo = __ldg(lv.boff + l);
    unsigned long long cnu = 0;
    for (int t0 = 0; t0 < T; t0 += PCH) {
        MaskT pm[PCH];
        unsigned long long fw[PCH];   // fingerprint word of each probe's group
        uint32_t hsv[PCH], fpv[PCH], valid = 0;
#pragma unroll
        for (int j = 0; j < PCH; ++j) {
            const int t = t0 + j;
            pm[j] = 0;
            fw[j] = ~0ull;
            hsv[j] = fpv[j] = 0;
            if (t < T) {
                const MaskT probe = t > 0 ? next_probe(t < T - 1) : (MaskT)0;
                pm[j] = probe;
                uint64_t hh;
                if (probe_hash(c, probe, hh)) {
                    hsv[j] = (uint32_t)hh & gmask;
                    fpv[j] = slot_fp(hh);
                    fw[j] = __ldg(slots + (uint64_t)hsv[j] * kGroupWords);
                    valid |= 1u << j;
                }
            }
        }
#pragma unroll
        for (int j = 0; j < PCH; ++j) {
            const int t = t0 + j;
            if (t >= T) break;
            int32_t res = -1;
            if (valid & (1u << j)) {
                unsigned long long w = fw[j];
                uint32_t h = hsv[j];
                bool done = false;
                for (uint32_t p = 0; p <= gmask && !done; ++p) {
                    const unsigned long long* grp = slots + (uint64_t)h * kGroupWords;
#pragma unroll
                    for (int e = 0; e < kGroupSlots && !done; ++e) {
                        const uint32_t f = (uint32_t)(w >> (16 * e)) & 0xFFFFu;
                        if (f == kEmptyFp) {
                            done = true;
                        } else if (f == fpv[j]) {
                            const uint32_t bj = __ldg(reinterpret_cast<const uint32_t*>(grp + 1) + e);
                            u128 k;
                            probe_key(c, pm[j], k);
                            if (key_matches(lv.ukeys + (bo + bj) * KW, k, KW)) {
                                res = (int32_t)bj;
                                done = true;
                            }
                        }
                    }
                    h = (h + 1) & gmask;
                    if (!done) w = __ldg(slots + (uint64_t)h * kGroupWords);
                }
            }
            qb[t] = res;
            if (res >= 0) cnu += __ldg(lv.sizes + bo + res);
        }
    }
    if (cnu) atomicAdd(a.cnu + q, cnu);
}

// Lookups of the split form. A thread takes kResolveSlots probe slots
// t = S*g .. S*g+S-1 of one (table, query) pair, queries fastest across
// threads, so that the hash and mask reads coalesce and S filter loads are in
// flight at once (eight measured fastest of 4, 8 and 16).
// Slots the enumeration marked -2 hold a valid probe: the key filter rules
// most absent keys out with one 4-byte load; otherwise the group walk of
// k_probe_fast runs, and a fingerprint match is verified against the key
// rebuilt from the pair's home key and sorted deltas (as probe_key does).
constexpr int kResolveSlots = 8;   // a multiple of 4
static_assert(kResolveSlots % 4 == 0, "slots per lookup thread");

__device__ __forceinline__ int32_t resolve_slot(const ProbeArgs& a, int l, int q, uint64_t hh, uint32_t pmask) {
    const LookupView& lv = a.lv;
    const int M = lv.M, KW = lv.KW;
    const uint32_t gmask = __ldg(lv.hmask + l);
    const unsigned long long* slots = lv.hslots + __ldg(lv.hoff + l);
    const uint64_t bo = __ldg(lv.boff + l);
    const uint32_t fp = slot_fp(hh);
    uint32_t h = (uint32_t)hh & gmask;
    bool have_key = false;
    u128 key = 0;
    for (uint32_t p = 0; p <= gmask; ++p) {
        const unsigned long long* grp = slots + (uint64_t)h * kGroupWords;
        const unsigned long long w = __ldg(grp);
        for (int e = 0; e < kGroupSlots; ++e) {
            const uint32_t f = (uint32_t)(w >> (16 * e)) & 0xFFFFu;
            if (f == kEmptyFp) return -1;
            if (f != fp) continue;
            if (!have_key) {
                const uint4* cx = a.pctx + ((int64_t)l * a.Q + q) * 3;
                const uint4 k0 = cx[0], e0 = cx[1], e1 = cx[2];
                uint32_t up = 0, dn = 0;
                for (uint32_t b = pmask; b; b &= b - 1) {
                    const int bit = lowest_bit(b);
                    const int wi = bit >> 2;
                    const uint32_t word = wi == 0 ? e0.x : wi == 1 ? e0.y : wi == 2 ? e0.z : wi == 3 ? e0.w
                                        : wi == 4 ? e1.x : wi == 5 ? e1.y : wi == 6 ? e1.z : e1.w;
                    const uint32_t en = (word >> (8 * (bit & 3))) & 0xFFu;
                    if (en & 0x80u) up |= 1u << (en & 0x3fu);
                    else dn |= 1u << (en & 0x3fu);
                }
                key = ((u128)k0.w << 96) | ((u128)k0.z << 64) | ((u128)k0.y << 32) | (u128)k0.x;
                const unsigned long long* funit = lv.funit + 2 * (int64_t)l * M;
                for (uint32_t b = up & ~dn; b; b &= b - 1) key += unit_of(funit, lowest_bit(b));
                for (uint32_t b = dn & ~up; b; b &= b - 1) key -= unit_of(funit, lowest_bit(b));
                have_key = true;
            }
            const uint32_t bj = __ldg(reinterpret_cast<const uint32_t*>(grp + 1) + e);
            if (key_matches(lv.ukeys + (bo + bj) * KW, key, KW)) return (int32_t)bj;
        }
        h = (h + 1) & gmask;
    }
    return -1;
}

__global__ void __launch_bounds__(256, 5) k_probe_resolve(const __grid_constant__ ProbeArgs a) {
    const LookupView& lv = a.lv;
    const int Q = a.Q, T = a.T;
    const int G = (T + kResolveSlots - 1) / kResolveSlots;
    const int64_t i = (int64_t)blockIdx.x * 256 + threadIdx.x;
    if (i >= (int64_t)lv.L * G * Q) return;
    const int q = (int)(i % Q);
    const int64_t lg = i / Q;
    const int l = (int)(lg / G), t0 = (int)(lg - (int64_t)l * G) * kResolveSlots;
    int32_t* qb = a.qbuckets + ((int64_t)l * Q + q) * T + t0;
    const bool vec = (T & 3) == 0;   // 16-byte accesses: every group of four slots lies within T
    int v[kResolveSlots];
#pragma unroll
    for (int c = 0; c < kResolveSlots; c += 4) {
        if (vec) {
            int4 x = make_int4(-1, -1, -1, -1);
            if (t0 + c < T) x = *reinterpret_cast<const int4*>(qb + c);
            v[c] = x.x;
            v[c + 1] = x.y;
            v[c + 2] = x.z;
            v[c + 3] = x.w;
        } else {
#pragma unroll
            for (int k = c; k < c + 4; ++k) v[k] = t0 + k < T ? qb[k] : -1;
        }
    }
    bool any = false;
#pragma unroll
    for (int k = 0; k < kResolveSlots; ++k) any |= v[k] == -2;
    if (!any) return;
    const int64_t base = (int64_t)l * T * Q + (int64_t)t0 * Q + q;
    // Filter words of the pending slots, all loads in flight together.
    const uint32_t* filt = lv.filt ? lv.filt + __ldg(lv.fl_off + l) : nullptr;
    const uint32_t fmask = lv.filt ? __ldg(lv.fl_mask + l) : 0;
    uint32_t fw[kResolveSlots], need[kResolveSlots];
#pragma unroll
    for (int k = 0; k < kResolveSlots; ++k) {
        need[k] = 0;
        fw[k] = 0;
        if (v[k] == -2) {
            const uint32_t fx = filter_mix(a.ph[base + (int64_t)k * Q]);
            need[k] = filter_bits(fx);
            fw[k] = filt ? __ldg(filt + (fx & fmask)) : ~0u;
        }
    }
    // Slots the filter rules out are misses; the rest (a few percent when
    // most probes miss) are resolved one at a time after the common store.
    uint32_t pass = 0;
#pragma unroll
    for (int k = 0; k < kResolveSlots; ++k) {
        if (v[k] != -2) continue;
        if ((fw[k] & need[k]) == need[k]) pass |= 1u << k;
        else v[k] = -1;
    }
#pragma unroll
    for (int c = 0; c < kResolveSlots; c += 4) {
        if (vec) {
            if (t0 + c < T) *reinterpret_cast<int4*>(qb + c) = make_int4(v[c], v[c + 1], v[c + 2], v[c + 3]);
        } else {
#pragma unroll
            for (int k = c; k < c + 4; ++k)
                if (t0 + k < T) qb[k] = v[k];
        }
    }
    if (!pass) return;
    unsigned long long added = 0;
    const uint64_t bo = __ldg(lv.boff + l);
#pragma unroll 1
    for (; pass; pass &= pass - 1) {
        const int k = lowest_bit(pass);
        const int32_t res = resolve_slot(a, l, q, a.ph[base + (int64_t)k * Q], a.pmask[base + (int64_t)k * Q]);
        qb[k] = res;
        if (res >= 0) added += __ldg(lv.sizes + bo + res);
    }
    if (added) atomicAdd(a.cnu + q, added);
}

template <typename MaskT, int PCH, int MM, int kForm>
cudaError_t launch_probe_fast_v(const ProbeArgs& a, cudaStream_t st) {
    const size_t smem = (size_t)PF * probe_fast_bytes_per_thread<MaskT>(a.lv.M, a.T, MM == 0);
    static std::atomic<size_t> cap{0};   // dynamic shared memory this kernel is opted into
    const cudaError_t e = opt_in_smem(k_probe_fast<MaskT, PCH, MM, kForm>, smem, cap);
    if (e != cudaSuccess) return e;
    const int64_t n = (int64_t)a.lv.L * a.Q;
    k_probe_fast<MaskT, PCH, MM, kForm><<<(unsigned)((n + PF - 1) / PF), PF, smem, st>>>(a);
    if (kForm == 1) {
        const int64_t threads = n * ((a.T + kResolveSlots - 1) / kResolveSlots);
        k_probe_resolve<<<(unsigned)((threads + 255) / 256), 256, 0, st>>>(a);
    }
    return cudaGetLastError();
}

template <typename MaskT, int MM>
cudaError_t launch_probe_fast_t(const ProbeArgs& a, cudaStream_t st) {
    if constexpr (sizeof(MaskT) == 4) {
        if (a.split == 2) return launch_probe_fast_v<MaskT, 1, MM, 2>(a, st);
        if (a.split) return launch_probe_fast_v<MaskT, 1, MM, 1>(a, st);
    }
    switch (a.pch) {
        case 1: return launch_probe_fast_v<MaskT, 1, MM, 0>(a, st);
        case 4: return launch_probe_fast_v<MaskT, 4, MM, 0>(a, st);
        default: return launch_probe_fast_v<MaskT, 2, MM, 0>(a, st);
    }
}

// 32-bit masks when the 2M sorted deltas fit (M <= 16), with the deltas
// ordered in registers for M padded to 8, 12 or 16; the split form exists
// for these. 64-bit masks (M <= 32) use the shared-memory ordering.
cudaError_t launch_probe_fast(const ProbeArgs& a, cudaStream_t st) {
    const int M = a.lv.M;
    if (M <= 8) return launch_probe_fast_t<uint32_t, 8>(a, st);
    if (M <= 12) return launch_probe_fast_t<uint32_t, 12>(a, st);
    if (M <= 16) return launch_probe_fast_t<uint32_t, 16>(a, st);
    ProbeArgs b = a;
    b.split = 0;
    return launch_probe_fast_t<uint64_t, 0>(b, st);
}

__global__ void __launch_bounds__(CT) k_candidates(CandArgs a) {
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ uint32_t s_ucount;
    __shared__ int s_ok;
    __shared__ unsigned long long s_off;
    __shared__ int s_wn[CW];
    __shared__ GatherSmem<CT, GCH> s_gather;

    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int q = a.qlist ? a.qlist[blockIdx.x] : (int)blockIdx.x;
    const int D = a.D, K = a.K, L = a.L, T = a.T;
    const int Dp = (D + 3) & ~3;
    float* qs = reinterpret_cast<float*>(smem);
    uint32_t* sh_set = reinterpret_cast<uint32_t*>(qs + Dp);
    uint32_t* sh_list = sh_set + SM_SLOTS;
    float* wd_all = reinterpret_cast<float*>(sh_list + SM_CAP);
    uint32_t* wi_all = reinterpret_cast<uint32_t*>(wd_all + CW * K);

    const unsigned long long C = a.cnu[q];
    int32_t* oid = a.out_ids + (int64_t)q * K;
    float* od = a.out_d + (int64_t)q * K;
    if (C == 0) {
        for (int k = tid; k < K; k += CT) {
            oid[k] = -1;
            od[k] = FLT_MAX;
        }
        if (tid == 0) a.cu[q] = 0;
        return;
    }

    uint32_t* hset = sh_set;
    uint32_t* ulist = sh_list;
    uint32_t cap = SM_SLOTS;
    if (C > (unsigned long long)SM_CAP) {
        unsigned long long c2 = 1;
        while (c2 < 2 * C) c2 <<= 1;
        if (tid == 0) {
            const unsigned long long need = c2 + C;
            const unsigned long long off = atomicAdd(a.arena_top, need);
            s_ok = off + need <= a.arena_words;
            s_off = off;
            if (!s_ok) a.deferred[atomicAdd(a.n_deferred, 1u)] = q;
        }
        __syncthreads();
        if (!s_ok) return;
        hset = a.arena + s_off;
        cap = (uint32_t)c2;
        ulist = hset + cap;
    }
    for (int i = tid; i < Dp; i += CT) qs[i] = i < D ? a.queries[(int64_t)q * D + i] : 0.0f;
    for (uint32_t i = tid; i < cap; i += CT) hset[i] = kEmpty32;
    if (tid == 0) s_ucount = 0;
    __syncthreads();

    // Gather every matched bucket's ids (duplicate probes included, as the
    // reference's candidate lists are) and deduplicate them.
    const uint32_t mask = cap - 1;
    const uint32_t lcap = C > (unsigned long long)SM_CAP ? (uint32_t)C : (uint32_t)SM_CAP;
    const BucketView bv{a.qbuckets, a.boff, a.starts, a.sizes, a.ids, a.N, L, T, a.Q};
    gather_bucket_ids<CT, GCH>(bv, q, s_gather,
                               [&](uint32_t id) { set_insert(hset, mask, ulist, lcap, &s_ucount, id); });
    __syncthreads();
    const uint32_t U = s_ucount;

    // Distances in the reference lane order, per-warp sorted top-K.
    float* wd = wd_all + warp * K;
    uint32_t* wi = wi_all + warp * K;
    int n = 0;
    float thr_d = FLT_MAX;
    uint32_t thr_i = 0;
    const bool vec = (D & 3) == 0;
    const int per = vec ? 16 : 4;   // candidates per warp iteration
    for (uint32_t base = warp * per; base < U; base += CW * per) {
        float dist = 0.f;
        uint32_t id = 0;
        bool own;
        if (vec) {
            const uint32_t ci = base + (lane >> 1);
            const int h = lane & 1;
            const bool valid = ci < U;
            id = valid ? ulist[ci] : 0u;
            const float* rowp = a.X + (int64_t)id * D;
            float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
            if (valid) {
                for (int c = 4 * h; c < D; c += 8) {
                    const float4 x = __ldg(reinterpret_cast<const float4*>(rowp + c));
                    const float4 qv = *reinterpret_cast<const float4*>(qs + c);
                    const float d0 = __fsub_rn(qv.x, x.x), d1 = __fsub_rn(qv.y, x.y);
                    const float d2 = __fsub_rn(qv.z, x.z), d3 = __fsub_rn(qv.w, x.w);
                    s0 = __fmaf_rn(d0, d0, s0);
                    s1 = __fmaf_rn(d1, d1, s1);
                    s2 = __fmaf_rn(d2, d2, s2);
                    s3 = __fmaf_rn(d3, d3, s3);
                }
            }
            const float o0 = __shfl_xor_sync(0xffffffffu, s0, 1), o1 = __shfl_xor_sync(0xffffffffu, s1, 1);
            const float o2 = __shfl_xor_sync(0xffffffffu, s2, 1), o3 = __shfl_xor_sync(0xffffffffu, s3, 1);
            const float t0 = __fadd_rn(s0, o0), t1 = __fadd_rn(s1, o1), t2 = __fadd_rn(s2, o2), t3 = __fadd_rn(s3, o3);
            dist = __fadd_rn(__fadd_rn(t0, t2), __fadd_rn(t1, t3));
            own = valid && h == 0;
        } else {
            const uint32_t ci = base + (lane >> 3);
            const int r = lane & 7;
            const bool valid = ci < U;
            id = valid ? ulist[ci] : 0u;
            const float* rowp = a.X + (int64_t)id * D;
            float s = 0.f;
            if (valid)
                for (int c = r; c < D; c += 8) {
                    const float df = __fsub_rn(qs[c], __ldg(rowp + c));
                    s = __fmaf_rn(df, df, s);
                }
            const float t = __fadd_rn(s, __shfl_xor_sync(0xffffffffu, s, 4));
            const float u = __fadd_rn(t, __shfl_xor_sync(0xffffffffu, t, 2));
            dist = __fadd_rn(u, __shfl_xor_sync(0xffffffffu, u, 1));
            own = valid && r == 0;
        }
        uint32_t want = __ballot_sync(0xffffffffu, own && lessp(dist, id, thr_d, thr_i));
        while (want) {
            const int src = __ffs(want) - 1;
            want &= want - 1;
            const float cdv = __shfl_sync(0xffffffffu, dist, src);
            const uint32_t cid = __shfl_sync(0xffffffffu, id, src);
            if (lessp(cdv, cid, thr_d, thr_i)) warp_insert(wd, wi, n, K, cdv, cid, thr_d, thr_i);
        }
    }
    if (lane == 0) s_wn[warp] = n;
    __syncthreads();
    if (warp == 0) {
        for (int w = 1; w < CW; ++w) {
            const int nw = s_wn[w];
            const float* od2 = wd_all + w * K;
            const uint32_t* oi2 = wi_all + w * K;
            for (int e = 0; e < nw; ++e) {
                const float d = od2[e];
                const uint32_t id = oi2[e];
                if (!lessp(d, id, thr_d, thr_i)) break;
                warp_insert(wd, wi, n, K, d, id, thr_d, thr_i);
            }
        }
        for (int k = lane; k < K; k += 32) {
            oid[k] = k < n ? (int32_t)wi[k] : -1;
            od[k] = k < n ? wd[k] : FLT_MAX;
        }
        if (lane == 0) {
            a.cu[q] = U;
            atomicAdd(a.totals + 0, (unsigned long long)U);
            atomicAdd(a.totals + 1, C);
        }
    }
}

}  // namespace

// Whether the fast kernel serves these arguments. It keeps per-thread state
// in shared memory: used while a block's slice stays within 100 KB (two
// blocks per SM), i.e. T <= 64 for M <= 16. CULSH_PROBE_GENERIC forces the
// general kernel (the tests run both).
static bool probe_fast_eligible(const ProbeArgs& a) {
    const bool generic_only = getenv("CULSH_PROBE_GENERIC") != nullptr;
    const size_t fast_bytes = (size_t)PF * (a.lv.M <= 16 ? probe_fast_bytes_per_thread<uint32_t>(a.lv.M, a.T)
                                                         : probe_fast_bytes_per_thread<uint64_t>(a.lv.M, a.T));
    return !generic_only && a.small_codes && a.lv.KW <= 4 && a.T <= 64 && a.lv.M <= 32 && fast_bytes <= 100 * 1024;
}

int probe_launches(const ProbeArgs& a) {
    if ((int64_t)a.lv.L * a.Q <= 0) return 0;
    return probe_fast_eligible(a) && a.split == 1 && a.lv.M <= 16 ? 2 : 1;
}

cudaError_t launch_probe(const ProbeArgs& a, cudaStream_t st) {
    const int64_t n = (int64_t)a.lv.L * a.Q;
    if (n <= 0) return cudaSuccess;
    if (probe_fast_eligible(a)) return launch_probe_fast(a, st);
    k_probe<<<(unsigned)((n + 127) / 128), 128, 0, st>>>(a);
    return cudaGetLastError();
}

int cand_smem_capacity() { return SM_CAP; }

size_t cand_arena_words(unsigned long long nonunique) {
    if (nonunique <= (unsigned long long)SM_CAP) return 0;
    unsigned long long c2 = 1;
    while (c2 < 2 * nonunique) c2 <<= 1;
    return (size_t)(c2 + nonunique);
}

cudaError_t launch_candidates(const CandArgs& a, cudaStream_t st) {
    const int nblk = a.qlist ? a.nq : a.Q;
    if (nblk <= 0) return cudaSuccess;
    const size_t smem = sizeof(float) * (size_t)((a.D + 3) & ~3) + sizeof(uint32_t) * (SM_SLOTS + SM_CAP) +
                        (size_t)CW * a.K * (sizeof(float) + sizeof(uint32_t));
    static std::atomic<size_t> cap{0};   // dynamic shared memory this kernel is opted into
    const cudaError_t e = opt_in_smem(k_candidates, smem, cap);
    if (e != cudaSuccess) return e;
    k_candidates<<<nblk, CT, smem, st>>>(a);
    return cudaGetLastError();
}

}  // namespace culsh
