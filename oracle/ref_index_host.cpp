// Entry points over the reference's own index-side host code (compiled in
// the same translation unit, after it: see ref_index_shim.h and the
// Makefile's `ref` target). Test infrastructure only: nothing in the library
// links or loads it.

extern "C" {

// codes: one table's floored code rows, N x M column-major (as the reference
// keeps them after projectMatrix + kernel_floorMatrix, cuLSH_Indexing.cu:215).
// Runs radixSortRows_1matrix + calculateBuckets (cuLSH_Indexing.cu:71-144):
// perm[N] gets the point ids in sorted row order (the table's totalIndices),
// starts/sizes[*nb] the bucket boundaries. Returns 0.
int ref_sort_buckets(const float* codes, int N, int M, unsigned* perm, unsigned* starts, unsigned* sizes,
                     unsigned* nb) {
    ThrustFloatD d_matrix(codes, codes + (size_t)N * M);
    ThrustUnsignedD d_perm;
    cuLSH::radixSortRows_1matrix(d_perm, d_matrix, N, M);
    ThrustUnsignedD d_idx, d_sizes;
    cuLSH::calculateBuckets(d_idx, d_sizes, d_matrix, N, M, d_perm);
    thrust::copy(d_perm.begin(), d_perm.end(), perm);
    thrust::copy(d_idx.begin(), d_idx.end(), starts);
    thrust::copy(d_sizes.begin(), d_sizes.end(), sizes);
    *nb = (unsigned)d_idx.size();
    return 0;
}

// HashTables::load(in), then HashTables::save(out) (cuLSH_HashTables.cu:395-483).
// Returns 0, or 1 / 2 when the load / the save fails.
int ref_load_save(const char* in, const char* out) {
    cuLSH::HashTables h;
    if (!h.load(in)) return 1;
    if (!h.save(out)) return 2;
    return 0;
}

}  // extern "C"
