// The reference propagation's queue: std::priority_queue<QueueItem> ordered by corrcoef, the
// smallest on top (reliability_propagation.cpp:44-53, 270-275).  Which of two equal keys comes out
// first is decided by the binary heap's layout, so this is that binary heap itself: on a push the
// new element rises past every parent with a larger key; on a pop the last element fills the
// root's place after the hole has been walked down to a leaf through, at each level, the right
// child unless the left one's key is smaller.  Keys K (a float table's keys are floats: the same
// order and the same ties) and points in separate arrays.  Host code only.
#pragma once

#include <cstddef>
#include <vector>

namespace tdic {

template <typename K>
struct TieHeap {
    std::vector<K> key;
    std::vector<int> val;
    size_t n = 0;
    bool empty() const { return n == 0; }
    int top() const { return val[0]; }
    void push(K k, int v) {
        if (n == key.size()) {
            key.resize(2 * n + 64);
            val.resize(2 * n + 64);
        }
        rise(n++, 0, k, v);
    }
    void pop() {
        if (n > 1) {
            const K k = key[n - 1];
            const int v = val[n - 1];
            key[n - 1] = key[0];
            val[n - 1] = val[0];
            const size_t len = n - 1;
            size_t hole = 0, child = 0;
            while (child < (len - 1) / 2) {
                child = 2 * (child + 1);
                if (key[child] > key[child - 1]) --child;
                key[hole] = key[child];
                val[hole] = val[child];
                hole = child;
            }
            if ((len & 1) == 0 && child == (len - 2) / 2) {
                child = 2 * (child + 1);
                key[hole] = key[child - 1];
                val[hole] = val[child - 1];
                hole = child - 1;
            }
            rise(hole, 0, k, v);
        }
        --n;
    }
    void rise(size_t hole, size_t top, K k, int v) {
        while (hole > top) {
            const size_t parent = (hole - 1) / 2;
            if (!(key[parent] > k)) break;
            key[hole] = key[parent];
            val[hole] = val[parent];
            hole = parent;
        }
        key[hole] = k;
        val[hole] = v;
    }
};

}  // namespace tdic
