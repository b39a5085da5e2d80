/*
 * cuLSH.h - drop-in replacement for the header of cuLSH (ariskag/cuLSH).
 *
 * Declares cuLSH::HashTables and cuLSH::SearchTables with the public members
 * of cuLSH_HashTables.cu:51-108 and cuLSH_SearchTables.cu:42-107, same names,
 * argument meaning and bool error convention (false + a message on stdout in
 * the style of the reference's DEF_PRINT_ERROR, cuLSH.h:79). The members are
 * inline wrappers over the C ABI of libculsh (culsh.h): include this header,
 * compile with g++ or nvcc, link with -lculsh.
 *
 * Differences from the reference, all deliberate:
 *  - copying the objects is disabled (the reference's shallow copies double-free);
 *  - reset(N,D,L,M,W) draws A and b from a seeded counter-based generator
 *    seeded with time(0) (the reference seeds cuRAND with time(0));
 *  - getKnnDistances() returns squared distances, exactly like the reference.
 */
#ifndef CULSH_GB300_DROPIN_H
#define CULSH_GB300_DROPIN_H

#include <climits>
#include <cstdio>
#include <ctime>

#include "culsh.h"

#define CULSH_DROPIN_ERROR(...)                                   \
    do {                                                          \
        printf("[Error @ %s, l.%d] ", __FILE__, __LINE__);        \
        printf(__VA_ARGS__);                                      \
    } while (0)

namespace cuLSH {

class HashTables {
   public:
    HashTables(void) : ix_(0) {
        if (culsh_index_create(&ix_) != CULSH_OK) ix_ = 0;
    }
    ~HashTables(void) { culsh_index_destroy(ix_); }
    HashTables(const HashTables&) = delete;
    HashTables& operator=(const HashTables&) = delete;

    // cuLSH_HashTables.cu:190-249
    bool reset(int N, int D, int L, int M, float W, FILE* debugStream = 0) {
        return check(culsh_index_reset_random(ix_, N, D, L, M, W, (unsigned long long)time(0), debugStream));
    }
    bool reset(int N, int D, int L, int M, float W, float** A, float** b, FILE* debugStream = 0) {
        return check(culsh_index_reset(ix_, N, D, L, M, W, (const float* const*)A, (const float* const*)b,
                                       debugStream));
    }
    bool reset(const char* filename, FILE* debugStream = 0) { return load(filename, debugStream); }

    // cuLSH_HashTables.cu:486-520
    bool index(const float* matrix, FILE* debugStream = 0) {
        return check(culsh_index_build(ix_, matrix, debugStream));
    }

    // cuLSH_HashTables.cu:89-103
    int getN(void) { return param(0); }
    int getD(void) { return param(1); }
    int getL(void) { return param(2); }
    int getM(void) { return param(3); }
    float getW(void) {
        float W = 0.0f;
        culsh_index_params(ix_, 0, 0, 0, 0, &W);
        return W;
    }
    const float* getA(int table) { return culsh_index_A(ix_, table); }
    const float* getb(int table) { return culsh_index_b(ix_, table); }
    unsigned getBuckets(int table) { return culsh_index_bucket_count(ix_, table); }
    const unsigned* getBuckets(void) { return culsh_index_bucket_counts(ix_); }
    const unsigned* getBuckets_totalIndices(int table) { return culsh_index_total_indices(ix_, table); }
    const unsigned* getBuckets_startingIndices(int table) { return culsh_index_starting_indices(ix_, table); }
    const unsigned* getBuckets_sizes(int table) { return culsh_index_sizes(ix_, table); }
    const float* getBuckets_codes(int table) { return culsh_index_codes(ix_, table); }

    // cuLSH_HashTables.cu:395-483
    bool save(const char* filename, FILE* debugStream = 0) {
        return check(culsh_index_save(ix_, filename, debugStream));
    }
    bool load(const char* filename, FILE* debugStream = 0) {
        return check(culsh_index_load(ix_, filename, debugStream));
    }

    culsh_index* handle(void) { return ix_; }

   private:
    culsh_index* ix_;
    int param(int which) {
        int v[4] = {0, 0, 0, 0};
        culsh_index_params(ix_, &v[0], &v[1], &v[2], &v[3], 0);
        return v[which];
    }
    static bool check(int rc) {
        if (rc == CULSH_OK) return true;
        CULSH_DROPIN_ERROR("%s\n", culsh_last_error());
        return false;
    }
};

class SearchTables {
   public:
    // cuLSH_SearchTables.cu:44-52
    typedef struct {
        float buckets;
        float collect;
        float sort;
        float unique;
        float distances;
        float knn;
        void reset(void) { buckets = collect = sort = unique = distances = knn = 0.0; }
    } timesStruct;

    SearchTables(void) : s_(0), ht_(0) {
        if (culsh_search_create(&s_) != CULSH_OK) s_ = 0;
    }
    ~SearchTables(void) { culsh_search_destroy(s_); }
    SearchTables(const SearchTables&) = delete;
    SearchTables& operator=(const SearchTables&) = delete;

    // cuLSH_SearchTables.cu:127-139
    void reset(HashTables* hashtables, int K, int T = 1) {
        ht_ = hashtables;
        culsh_search_reset(s_, hashtables ? hashtables->handle() : 0, K, T);
    }

    // cuLSH_SearchTables.cu:197-463
    bool search(const float* queries, const int Q, const float* dataset, FILE* debugStream = 0) {
        const int rc = culsh_search_run(s_, queries, Q, dataset, debugStream);
        if (rc == CULSH_OK) return true;
        CULSH_DROPIN_ERROR("%s\n", culsh_last_error());
        return false;
    }

    // cuLSH_SearchTables.cu:83-105
    float getSelectivity(void) { return culsh_search_selectivity(s_); }
    float getNonUniquePercentage(void) { return culsh_search_nonunique_percentage(s_); }
    const int* getQueryBuckets(int table) { return culsh_search_query_buckets(s_, table); }
    unsigned getTotalCandidates_unique(void) { return sat(culsh_search_total_unique(s_)); }
    unsigned getTotalCandidates_nonUnique(void) { return sat(culsh_search_total_nonunique(s_)); }
    const int* getKnnIds(void) { return culsh_search_knn_ids(s_); }
    const float* getKnnDistances(void) { return culsh_search_knn_distances(s_); }
    void getTimes(timesStruct* times) {
        culsh_times t;
        culsh_search_times(s_, &t);
        times->buckets = t.buckets;
        times->collect = t.collect;
        times->sort = t.sort;
        times->unique = t.unique;
        times->distances = t.distances;
        times->knn = t.knn;
    }

    culsh_search* handle(void) { return s_; }

   private:
    culsh_search* s_;
    HashTables* ht_;
    static unsigned sat(unsigned long long v) { return v > UINT_MAX ? UINT_MAX : (unsigned)v; }
};

}  // namespace cuLSH

#endif /* CULSH_GB300_DROPIN_H */
