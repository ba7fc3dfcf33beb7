// Sorting a block's tile of work items by code path, so that the lanes of a
// warp take the same branches (used by the Jacobian and flash-derivative
// kernels).
#pragma once

namespace ocpx {

// A stable counting sort of a tile of n items by class (key_of(i) < CLASSES)
// in shared memory (key_s and idx_s hold n entries, n <= 65,536): idx_s[0..n)
// lists the items class by class, each class in item order.  Within a chunk of blockDim.x items, lanes of one
// class rank by lane (match_any) and warps take their offsets in turn.  All
// threads of the block call it.
template <int CLASSES, class KeyOf>
__device__ void tile_sort(int n, KeyOf key_of, unsigned* cnt, unsigned short* key_s, unsigned short* idx_s)
{
    static_assert(CLASSES % 32 == 0, "classes in whole warps");
    const int t = threadIdx.x;
    for (int k = t; k < CLASSES; k += blockDim.x) cnt[k] = 0;
    __syncthreads();
    for (int i = t; i < n; i += blockDim.x) {
        const int key = key_of(i);
        key_s[i] = (unsigned short)key;
        atomicAdd(&cnt[key], 1u);
    }
    __syncthreads();
    if (t < 32) {  // exclusive scan of the class counts, CLASSES / 32 per lane
        constexpr int PER = CLASSES / 32;
        unsigned part = 0;
        for (int k = 0; k < PER; k++) part += cnt[t * PER + k];
        unsigned incl = part;
        for (int d = 1; d < 32; d <<= 1) {
            const unsigned v = __shfl_up_sync(0xffffffffu, incl, d);
            if (t >= d) incl += v;
        }
        unsigned run = incl - part;
        for (int k = 0; k < PER; k++) {
            const unsigned v = cnt[t * PER + k];
            cnt[t * PER + k] = run;
            run += v;
        }
    }
    __syncthreads();
    const unsigned lane = t & 31, warp = t >> 5, nwarps = blockDim.x >> 5;
    for (int base = 0; base < n; base += blockDim.x) {
        const int i = base + t;
        const bool valid = i < n;
        const unsigned key = valid ? key_s[i] : 0xffffu;
        const unsigned peers = __match_any_sync(0xffffffffu, key);
        const unsigned rank = __popc(peers & ((1u << lane) - 1u));
        unsigned off = 0;
        for (unsigned w = 0; w < nwarps; w++) {
            if (w == warp && valid && rank == 0) {
                off = cnt[key];
                cnt[key] = off + __popc(peers);
            }
            __syncthreads();
        }
        off = __shfl_sync(0xffffffffu, off, __ffs(peers) - 1);
        if (valid) idx_s[off + rank] = (unsigned short)i;
    }
    __syncthreads();
}

}  // namespace ocpx
