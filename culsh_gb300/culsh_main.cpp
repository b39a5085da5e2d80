// Command-line index + search over a raw float32 data file, the counterpart
// of the reference's demo program (cuLSH_main.cu:21-108), written against the
// drop-in header so that it exercises the same calls a user program makes.
//
//   culsh_main [filename] [D] [N] [L] [M] [W] [Q] [K] [T]
//
// The file holds N points of D floats each (point-contiguous, the layout
// HashTables::index takes). The queries are the first Q points. The
// projections are random (HashTables::reset(N, D, L, M, W), seeded from the
// clock as in the reference). Index and search times are wall-clock seconds
// around index() and search(); the per-stage times are getTimes().
//
// Differences from the demo, none of which change a result:
//  * times are printed with millisecond resolution (the demo prints whole
//    seconds of time(0));
//  * Q > N is rejected (the demo copies Q points out of an N-point buffer);
//  * if CULSH_SAVE_INDEX names a path, the built index is saved there with
//    HashTables::save (the reference's file layout), so that a run can be
//    inspected or reloaded later.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "cuLSH.h"

namespace {

double seconds_since(std::chrono::steady_clock::time_point t0) {
    return std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
}

}  // namespace

int main(int argc, char** argv) {
    if (argc != 10) {
        printf("%d given arguments, while %d are required...\n", argc, 9);
        printf("Arguments: [filename] [D] [N] [L] [M] [W] [Q] [K] [T]\n");
        return 0;
    }
    FILE* fp = fopen(argv[1], "rb");
    if (!fp) {
        printf("Could not open file with data matrix...\n");
        return 1;
    }
    const int D = atoi(argv[2]), N = atoi(argv[3]), L = atoi(argv[4]), M = atoi(argv[5]);
    const float W = (float)atof(argv[6]);
    const int Q = atoi(argv[7]), K = atoi(argv[8]), T = atoi(argv[9]);
    printf("data: [%d x %d], queries: [%d x %d], (L, M, W) = (%d, %d, %.2f), (Q, K, T) = (%d, %d, %d)\n", D, N, D,
           Q, L, M, W, Q, K, T);
    if (D <= 0 || N <= 0 || Q <= 0 || Q > N) {
        printf("Invalid sizes: need D > 0, N > 0 and 0 < Q <= N...\n");
        fclose(fp);
        return 1;
    }
    std::vector<float> dataset((size_t)D * N);
    const size_t got = fread(dataset.data(), sizeof(float), dataset.size(), fp);
    fclose(fp);
    if (got != dataset.size()) {
        printf("Could not load data matrix from file...\n");
        return 1;
    }
    std::vector<float> queries(dataset.begin(), dataset.begin() + (size_t)D * Q);

    cuLSH::HashTables hashtables;
    cuLSH::SearchTables searchtables;
    if (!hashtables.reset(N, D, L, M, W, stdout)) {
        printf("Could not reset tables...\n");
        return 1;
    }
    searchtables.reset(&hashtables, K, T);

    auto t0 = std::chrono::steady_clock::now();
    if (!hashtables.index(dataset.data(), stdout)) {
        printf("Failed to perform indexing...\n");
        return 1;
    }
    const double t_index = seconds_since(t0);
    printf("\n%.3f seconds to index\n\n", t_index);
    if (const char* path = getenv("CULSH_SAVE_INDEX")) {
        if (!hashtables.save(path)) {
            printf("Could not save the index to %s...\n", path);
            return 1;
        }
    }

    t0 = std::chrono::steady_clock::now();
    if (!searchtables.search(queries.data(), Q, dataset.data(), stdout)) {
        printf("Failed to perform searching...\n");
        return 1;
    }
    const double t_search = seconds_since(t0);
    printf("\n%.3f seconds to search\n\n", t_search);

    cuLSH::SearchTables::timesStruct times;
    searchtables.getTimes(&times);
    printf("%.3f seconds to index\n", t_index);
    printf("%.3f seconds to search\n", t_search);
    printf("\tCollecting: %f\n", times.collect);
    printf("\tSorting:    %f\n", times.sort);
    printf("\tUnique:     %f\n", times.unique);
    printf("\tDistances:  %f\n", times.distances);
    printf("\tnn indices: %f\n", times.knn);
    printf("Selectivity = %.3f%%\n", searchtables.getSelectivity());
    printf("Duplicate candidates = %.3f%%\n", searchtables.getNonUniquePercentage());
    return 0;
}
