// Per-query candidate heap of the tensor-core kNN epilogue (knn_tc.cu).
//
// A 4-ary max-heap of (squared distance, index) entries: the root is the largest kept
// distance, i.e. the current threshold once the heap holds C entries.  Four children per node
// halve the depth of a binary heap (4 levels for C = 120 instead of 7), and the children of a
// level are independent loads, so a replacement costs about four dependent shared-memory
// round trips.  Each entry is one 8-byte word (distance and index together), so moving an
// entry up is one load and one store.  Entry e of a heap lives at base[e * stride]: with the
// heaps of 32 lanes interleaved (stride = lanes per block, lane offset r), a warp's accesses
// to arbitrary entries stay bank-conflict free.
#pragma once

#include <cstdint>

#ifdef __CUDACC__
#define KNN_HEAP_HD __host__ __device__ __forceinline__
#else
#define KNN_HEAP_HD inline
#endif

namespace fitsne {

struct alignas(8) HeapEntry {
    float d;
    uint32_t i;
};

template <int kStride>
struct Heap4 {
    HeapEntry *h;  // this heap's entry 0
    KNN_HEAP_HD HeapEntry &at(int e) const { return h[e * kStride]; }
    KNN_HEAP_HD float top() const { return h[0].d; }

    // adds (v, id) to a heap of n < capacity entries (sift up)
    KNN_HEAP_HD void push(int &n, float v, uint32_t id) const {
        int pos = n++;
        while (pos > 0) {
            const int par = (pos - 1) >> 2;
            const HeapEntry p = at(par);
            if (p.d >= v) break;
            at(pos) = p;
            pos = par;
        }
        at(pos) = HeapEntry{v, id};
    }

    // places (v, id) at pos of a heap of n entries and sifts it down (replacing the root when
    // pos = 0)
    KNN_HEAP_HD void sift_down(int n, int pos, float v, uint32_t id) const {
        while (true) {
            const int c = 4 * pos + 1;
            if (c >= n) break;
            HeapEntry m = at(c);
            int mi = c;
            if (c + 3 < n) {  // four children: a two-round tournament
                const HeapEntry e1 = at(c + 1), e2 = at(c + 2), e3 = at(c + 3);
                const bool b01 = e1.d > m.d, b23 = e3.d > e2.d;
                const HeapEntry m01 = b01 ? e1 : m, m23 = b23 ? e3 : e2;
                const int i01 = b01 ? c + 1 : c, i23 = b23 ? c + 3 : c + 2;
                const bool b = m23.d > m01.d;
                m = b ? m23 : m01;
                mi = b ? i23 : i01;
            } else {
                for (int k = 1; k < 3 && c + k < n; ++k) {
                    const HeapEntry e = at(c + k);
                    if (e.d > m.d) {
                        m = e;
                        mi = c + k;
                    }
                }
            }
            if (m.d <= v) break;
            at(pos) = m;
            pos = mi;
        }
        at(pos) = HeapEntry{v, id};
    }

    // sift_down from the root without branches: the new root (v, id) of a heap of n <= 341
    // entries (four levels of children) goes down four fixed levels, children past n and
    // every level below the one where the entry stops predicated off, with sift_down's choice
    // of child.  The lanes of a warp stay together whatever depth their entries reach.
    KNN_HEAP_HD void replace_top(int n, float v, uint32_t id) const {
        const HeapEntry lowest{-3.402823466e38f, 0u};  // below every distance: never moves up
        int pos = 0;
        bool go = true;
#pragma unroll
        for (int l = 0; l < 4; ++l) {
            const int c = 4 * pos + 1;
            const HeapEntry e0 = (go && c < n) ? at(c) : lowest;
            const HeapEntry e1 = (go && c + 1 < n) ? at(c + 1) : lowest;
            const HeapEntry e2 = (go && c + 2 < n) ? at(c + 2) : lowest;
            const HeapEntry e3 = (go && c + 3 < n) ? at(c + 3) : lowest;
            const bool b01 = e1.d > e0.d, b23 = e3.d > e2.d;
            const HeapEntry m01 = b01 ? e1 : e0, m23 = b23 ? e3 : e2;
            const int i01 = b01 ? c + 1 : c, i23 = b23 ? c + 3 : c + 2;
            const bool b = m23.d > m01.d;
            const HeapEntry m = b ? m23 : m01;
            const bool mv = m.d > v;
            if (mv) at(pos) = m;
            pos = mv ? (b ? i23 : i01) : pos;
            go = mv;
        }
        at(pos) = HeapEntry{v, id};
    }

    // sorts the n entries ascending in place (heap sort)
    KNN_HEAP_HD void sort_ascending(int n) const {
        for (int end = n - 1; end > 0; --end) {
            const HeapEntry last = at(end);
            at(end) = at(0);
            sift_down(end, 0, last.d, last.i);
        }
    }
};

}  // namespace fitsne
