// Host check of the tensor-core kNN's candidate heap (fit-sne_gb300/csrc/knn_heap.cuh): for
// random streams with many equal distances, capacities 1..130 and interleaved storage, the
// heap fed through the epilogue's protocols (push until full, then replace the root when a
// distance is below it, with sift_down or replace_top; and the same through a queue of up to
// five candidates that passed a stale threshold, flushed when it would overflow) ends with
// the C smallest distances, sorted, each with its own index.
#include <algorithm>
#include <cstdio>
#include <random>
#include <utility>
#include <vector>

#include "../fit-sne_gb300/csrc/knn_heap.cuh"

using fitsne::Heap4;
using fitsne::HeapEntry;

int main() {
    std::mt19937 rng(12345);
    for (int trial = 0; trial < 3000; ++trial) {
        const int C = 1 + (int) (rng() % 130);
        const int M = (int) (rng() % 1500);
        std::vector<HeapEntry> mem((size_t) C * 4 + 4);
        const Heap4<4> hp{mem.data() + trial % 4};
        const int mode = trial % 3;  // 0: sift_down, 1: replace_top, 2: queued replace_top
        int n = 0;
        float thr = 3.4e38f;
        std::vector<std::pair<float, unsigned>> all;
        auto insert = [&](float d, unsigned i) {
            if (d < thr) {
                if (n < C) {
                    hp.push(n, d, i);
                    if (n == C) thr = hp.top();
                } else {
                    if (mode == 0)
                        hp.sift_down(n, 0, d, i);
                    else
                        hp.replace_top(n, d, i);
                    thr = hp.top();
                }
            }
        };
        std::vector<std::pair<float, unsigned>> queue;
        for (int k = 0; k < M; ++k) {
            const float d = (float) (rng() % 400) / 7.0f;
            all.push_back({d, (unsigned) k});
            if (mode < 2) {
                insert(d, (unsigned) k);
            } else if (d < thr) {
                if (queue.size() == 5) {
                    for (auto &e : queue) insert(e.first, e.second);
                    queue.clear();
                }
                queue.push_back({d, (unsigned) k});
            }
        }
        for (auto &e : queue) insert(e.first, e.second);
        hp.sort_ascending(n);
        std::vector<float> want;
        for (auto &p : all) want.push_back(p.first);
        std::sort(want.begin(), want.end());
        if (n != std::min(C, M)) {
            std::printf("trial %d: %d entries, expected %d\n", trial, n, std::min(C, M));
            return 1;
        }
        for (int e = 0; e < n; ++e) {
            const HeapEntry en = hp.at(e);
            if (en.d != want[e] || all[en.i].first != en.d) {
                std::printf("trial %d (C %d, M %d): entry %d = (%g, %u), expected distance %g\n", trial, C, M, e,
                            en.d, en.i, want[e]);
                return 1;
            }
        }
    }
    std::printf("ok\n");
    return 0;
}
