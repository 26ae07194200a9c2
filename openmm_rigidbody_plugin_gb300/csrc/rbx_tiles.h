// rbx_tiles.h -- the step kernel's block -> tile map, a pure function shared by the device and the
// host-side tests.
#pragma once

#ifdef __CUDACC__
#define RBX_HD __host__ __device__
#else
#define RBX_HD
#endif

namespace rbx {

// Tile of grid block i: the body tile (>= 0) or -1 - the free-atom tile. Free-atom tiles are spread
// over the grid in proportion rather than placed after the body tiles, where their FP64 velocity
// arithmetic (then used in mixed precision) queued on GB300's narrow FP64 pipe as a tail at the end
// of the grid: 100,000 free atoms cost 15 us of a 0.144 ms step, for 2 % of its bytes. Interleaved,
// that work overlaps the body tiles' memory traffic (0.1437 -> 0.1383 ms). Block i is a free-atom
// tile when c(i) = floor((i + 1) nf / T) (T = body + free-atom tiles) steps up there, so free-atom
// tile j runs right after the body tiles that cover the same span of slots (both are in slot
// order). Since nf <= T, c never steps by more than one, which makes the map a bijection from
// [0, T) onto [0, body tiles) and [0, free-atom tiles).
RBX_HD inline int tile_of_block(int i, int n_body_tiles, int n_free_tiles) {
    if (n_free_tiles == 0) return i;
    const long long T = (long long)n_body_tiles + n_free_tiles;
    const int c = (int)(((long long)i + 1) * n_free_tiles / T), c0 = (int)((long long)i * n_free_tiles / T);
    return c > c0 ? -c : i - c;
}

}  // namespace rbx
