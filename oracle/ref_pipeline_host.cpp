// Entry point over the reference's whole index and search path, compiled in
// the same translation unit after it (see ref_pipeline_shim.h and the
// Makefile's `ref` target). Test infrastructure only: nothing in the library
// links or loads it.

thread_local ref_dim3 threadIdx, blockIdx, blockDim, gridDim;
thread_local void (*ref_sync_hook)() = nullptr;
thread_local std::barrier<>* ref_block_barrier = nullptr;
void ref_block_sync() { ref_block_barrier->arrive_and_wait(); }

size_t ref_free_bytes = (size_t)1 << 40;

// The oracle's projection (oracle.cpp): with b = 0 and W = 1 it returns the
// bare canonical FMA chains, fl(fl(C - 0) / 1) = C.
extern "C" void oracle_project(const float* X, int64_t n_pts, int D, const float* A, const float* b, int L, int M,
                               float W, float* out);

// The reference's one GEMM (cuLSH_Indexing.cu:43-51): C (m x n, ldc = m) =
// op(A)' B with A the D x m data (lda = k = D) and B the D x n projection
// (ldb = D), alpha 1, beta 0. Any other form is refused.
cublasStatus_t cublasSgemm(cublasHandle_t, cublasOperation_t ta, cublasOperation_t tb, int m, int n, int k,
                           const float* alpha, const float* A, int lda, const float* B, int ldb, const float* beta,
                           float* C, int ldc) {
    if (ta != CUBLAS_OP_T || tb != CUBLAS_OP_N || lda != k || ldb != k || ldc != m || *alpha != 1.0f ||
        *beta != 0.0f)
        return CUBLAS_STATUS_NOT_SUPPORTED;
    std::vector<float> zero((size_t)n, 0.0f);
    oracle_project(A, m, k, B, zero.data(), 1, n, 1.0f, C);
    return CUBLAS_STATUS_SUCCESS;
}

extern "C" {

// HashTables::reset(N, D, L, M, W, A, b) + index(X), then SearchTables::reset
// (K, T) + search(queries, Q, X) (cuLSH_HashTables.cu:213-240,486-520,
// cuLSH_SearchTables.cu:127-139,197-463), as cuLSH_main.cu drives them.
//   X [N][D], A [L][M][D] (A[l] the reference's D x M column-major), b [L][M],
//   queries [Q][D]; free_bytes: what cuMemGetInfo reports (0: 1 TiB).
// Outputs (index packed as the oracle packs it): buckets[L]; ids, starts,
// sizes at l*N; codes at l*N*M with column stride buckets[l]; qbuckets
// [L][Q*T]; knn_ids / knn_d [Q][K]; totals = {non-unique, unique}.
// Returns 0, or 1 / 2 / 3 when the reset / index / search fails.
int ref_pipeline(const float* X, int N, int D, int L, int M, float W, const float* A, const float* b,
                 const float* queries, int Q, int K, int T, unsigned long long free_bytes, unsigned* buckets,
                 unsigned* ids, unsigned* starts, unsigned* sizes, float* codes, int* qbuckets, int* knn_ids,
                 float* knn_d, unsigned* totals) {
    ref_free_bytes = free_bytes ? (size_t)free_bytes : (size_t)1 << 40;
    std::vector<float*> Ap((size_t)L), bp((size_t)L);
    for (int l = 0; l < L; ++l) {
        Ap[l] = const_cast<float*>(A + (size_t)l * M * D);
        bp[l] = const_cast<float*>(b + (size_t)l * M);
    }
    cuLSH::HashTables h;
    if (!h.reset(N, D, L, M, W, Ap.data(), bp.data())) return 1;
    if (!h.index(X)) return 2;
    for (int l = 0; l < L; ++l) {
        const unsigned B = h.getBuckets(l);
        buckets[l] = B;
        std::memcpy(ids + (size_t)l * N, h.getBuckets_totalIndices(l), sizeof(unsigned) * N);
        std::memcpy(starts + (size_t)l * N, h.getBuckets_startingIndices(l), sizeof(unsigned) * B);
        std::memcpy(sizes + (size_t)l * N, h.getBuckets_sizes(l), sizeof(unsigned) * B);
        std::memcpy(codes + (size_t)l * N * M, h.getBuckets_codes(l), sizeof(float) * B * M);
    }
    cuLSH::SearchTables s;
    s.reset(&h, K, T);
    if (!s.search(queries, Q, X)) return 3;
    for (int l = 0; l < L; ++l) std::memcpy(qbuckets + (size_t)l * Q * T, s.getQueryBuckets(l), sizeof(int) * Q * T);
    std::memcpy(knn_ids, s.getKnnIds(), sizeof(int) * Q * K);
    std::memcpy(knn_d, s.getKnnDistances(), sizeof(float) * Q * K);
    totals[0] = s.getTotalCandidates_nonUnique();
    totals[1] = s.getTotalCandidates_unique();
    return 0;
}

}  // extern "C"
