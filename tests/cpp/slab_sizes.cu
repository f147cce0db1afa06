// Prints the split build's slab sizing (host side of the shared header): the
// constants, then for every chunk size built as slabs (17 .. kSlabMaxCells
// cells per edge) N, layers per slab, slabs per chunk, slab workspace bytes,
// the slab's vertex bound and the z-table bytes of a 16-octave fast build.
#include <cstdio>

#include "uww_internal.h"

int main()
{
    using namespace uww;
    std::printf("%d %u %u %d %u\n", kSlabThreads, kSlabBudget, kSlabActCap, kSlabMaxCells,
                chunk_layout(16).total);
    for (int N = 17; N <= kSlabMaxCells; ++N) {
        const int K = slab_layers(N);
        std::printf("%d %d %d %u %lld %zu\n", N, K, slab_count(N), slab_layout(N).total, slab_vertex_bound(N, K),
                    ztable_bytes(N + 1, UWW_MAX_OCTAVES));
    }
    return 0;
}
