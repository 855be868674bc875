// Test helper (host code only, no GPU needed): runs the engine's host ordering
// of long CSC columns (Engine::sort_long_columns,
// sovereign-solver_gb300/csrc/engine_impl.cuh) on a column range read from a
// binary file and writes the entries back, for tests/test_column_order.py.
//
// usage:  colsort_dump in.bin out.bin
// input:  int32 n, int32 j0, int32 j1, int32 cptr[n+1],
//         int32 idx[cptr[j1]-cptr[j0]], double val[cptr[j1]-cptr[j0]]
// output: int32 idx[...], double val[...] after ordering
#include "engine_impl.cuh"

#include <cstdio>

using namespace sps;

static bool read_all(FILE* f, void* p, size_t size, size_t count) { return fread(p, size, count, f) == count; }

int main(int argc, char** argv) {
    if (argc != 3) return 2;
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 3;
    int32_t n = 0, j0 = 0, j1 = 0;
    bool ok = read_all(f, &n, 4, 1) && read_all(f, &j0, 4, 1) && read_all(f, &j1, 4, 1);
    if (!ok || n < 0 || j0 < 0 || j1 < j0 || j1 > n) return 4;
    std::vector<int32_t> cptr(n + 1);
    ok = read_all(f, cptr.data(), 4, n + 1);
    const int64_t len = ok ? (int64_t)cptr[j1] - cptr[j0] : 0;
    std::vector<int32_t> idx(len);
    std::vector<double> val(len);
    ok = ok && read_all(f, idx.data(), 4, len) && read_all(f, val.data(), 8, len);
    fclose(f);
    if (!ok) return 4;
    if (j1 > j0) Engine<float>::sort_long_columns(cptr.data(), j0, j1, idx.data(), val.data());
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 5;
    fwrite(idx.data(), 4, len, o);
    fwrite(val.data(), 8, len, o);
    fclose(o);
    return 0;
}
