"""Line-by-line Python transliteration of the reference's multiprobe and top-K
kernels, used only to cross-check the C++ oracle.

It follows the control flow of cuLSH_Kernels.cu statement by statement
(kernel_calculateDeltas :266-289, balanceHeap_deltas :144-175,
kernel_calculateProbingCodes :188-257, balanceHeap_knnIds :356-398,
kernel_configureIds :406-433, kernel_sortIds :439-456) with float32 scalar
arithmetic, so that the oracle's independent C++ restatement can be compared
against a second reading of the same code. Pure Python loops: small cases only.
The one deliberate difference: 64-bit probe masks (the reference's 32-bit
``1 << i`` is undefined for i >= 31).
"""

from __future__ import annotations

import math

import numpy as np

F32 = np.float32
FLT_MAX = F32(np.finfo(np.float32).max)


def calculate_deltas(v):
    """cuLSH_Kernels.cu:266-289 for one query: floored codes and 2M deltas."""
    M = len(v)
    floored = [F32(math.floor(F32(x))) for x in v]
    deltas = [F32(0)] * (2 * M)
    for pos in range(M):
        value_non_floored = F32(v[pos])
        value_floored = floored[pos]
        delta_down = F32(value_non_floored - value_floored)
        delta_up = F32(F32(1) - delta_down)
        deltas[pos] = delta_down
        deltas[pos + M] = delta_up
    return floored, deltas


def balance_heap_deltas(permutation, deltas, total, total_levels):
    parent = 0
    for _level in range(total_levels - 1):
        left = parent * 2 + 1
        right = left + 1
        max_index = parent
        if left < total and permutation[left] == -1:
            max_index = left
        elif right < total and permutation[right] == -1:
            max_index = right
        else:
            if left < total and deltas[permutation[left]] > deltas[permutation[max_index]]:
                max_index = left
            if right < total and deltas[permutation[right]] > deltas[permutation[max_index]]:
                max_index = right
        if max_index == parent:
            break
        permutation[parent], permutation[max_index] = permutation[max_index], permutation[parent]
        parent = max_index


def _levels(x):
    # __float2int_ru(log2f(x)) for the small positive integers used here.
    return int(math.ceil(math.log2(x) - 1e-12))


def probing_codes(v, T):
    """Rows [T][M] of probe codes (row 0 = home code) for one query/table."""
    M = len(v)
    home, deltas = calculate_deltas(v)
    rows = [list(home)]
    if T <= 1:
        return np.array(rows, np.float32)
    total_levels = _levels(2 * M + 1)
    max_t = min(2 * M, 64)
    perm = [-1] * 64
    for i in range(2 * M):
        if perm[0] == -1 or deltas[i] < deltas[perm[0]]:
            perm[0] = i
            balance_heap_deltas(perm, deltas, max_t, total_levels)
    for i in range(max_t - 1, 0, -1):
        perm[0], perm[i] = perm[i], perm[0]
        balance_heap_deltas(perm, deltas, i, total_levels)
    combinations = [0] * T
    combinations_deltas = [F32(0)] * T
    combinations[0] = 1
    combinations_deltas[0] = deltas[perm[0]]
    size = 1
    max_perm_index = 0
    for t in range(1, T):
        min_value = FLT_MAX
        min_index = 0
        for i in range(size):
            value = combinations_deltas[i]
            if value < min_value:
                min_index = i
                min_value = value
        probe = combinations[min_index]
        maxt = probe.bit_length()
        row = list(rows[0])
        for i in range(maxt):
            if probe & (1 << i):
                row[perm[i] % M] = F32(row[perm[i] % M] + (F32(1) if perm[i] >= M else F32(-1)))
                max_perm_index = i
        rows.append(row)
        if max_perm_index < max_t - 1:
            probe |= 1 << (max_perm_index + 1)
            min_value = F32(min_value + deltas[perm[max_perm_index + 1]])
            combinations[min_index] = probe
            combinations_deltas[min_index] = min_value
            probe -= 1 << max_perm_index
            min_value = F32(min_value - deltas[perm[max_perm_index]])
            combinations[size] = probe
            combinations_deltas[size] = min_value
            size += 1
    return np.array(rows, np.float32)


def balance_heap_knn(heap, knn_ids, size, total_levels):
    parent = 0
    for _level in range(total_levels - 1):
        left = parent * 2 + 1
        right = left + 1
        max_index = parent
        if left < size:
            diff = F32(heap[left] - heap[parent])
            if diff >= 0 and (diff > 0 or knn_ids[left] > knn_ids[parent]):
                max_index = left
        if right < size:
            diff = F32(heap[right] - heap[max_index])
            if diff >= 0 and (diff > 0 or knn_ids[right] > knn_ids[max_index]):
                max_index = right
        if max_index == parent:
            break
        heap[parent], heap[max_index] = heap[max_index], heap[parent]
        knn_ids[parent], knn_ids[max_index] = knn_ids[max_index], knn_ids[parent]
        parent = max_index


def reference_topk(cand, dist, K):
    """kernel_configureIds + kernel_sortIds for one query (cand ascending)."""
    heap = [FLT_MAX] * K
    knn = [-1] * K
    total_levels = _levels(K + 1)
    for i in range(len(cand) - 1, -1, -1):
        qd = F32(dist[i])
        if qd < heap[0]:
            heap[0] = qd
            knn[0] = int(cand[i])
            balance_heap_knn(heap, knn, K, total_levels)
    for i in range(K - 1, 0, -1):
        heap[0], heap[i] = heap[i], heap[0]
        knn[0], knn[i] = knn[i], knn[0]
        balance_heap_knn(heap, knn, i, _levels(i + 1))
    return np.array(knn, np.int32), np.array(heap, np.float32)
