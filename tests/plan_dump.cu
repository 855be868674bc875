// Test helper (host code only, no GPU needed): runs the engine's row plan
// (SLAB choice + bin layout, sovereign-solver_gb300/csrc/engine_impl.cuh) on
// a problem read from a binary file and writes the plan back out, for
// tests/test_plan_layout.py.
//
// usage:  plan_dump in.bin out.bin block_cap [cols]
// input:  int32 m, int32 n, int64 nnz, int32 ptr[m+1], int32 idx[nnz],
//         int8 kind[m], int32 inv_col[n]
// output: a sequence of (int64 count, int32 data[count]) arrays:
//         slab flags, perm, fptr, soff, unit descriptors, bins (nbins,
//         total_blocks, then 12 ints per bin), totals (total, ntickets,
//         nslots, nslab_units)
#include "engine_impl.cuh"

#include <cstdio>
#include <cstdlib>

using namespace sps;

static bool read_all(FILE* f, void* p, size_t size, size_t count) { return fread(p, size, count, f) == count; }

int main(int argc, char** argv) {
    // optional 4th argument "cols": the column plan as the engine makes it
    // (one kind, no SLAB choice: make_plan(lens, nullptr, nullptr, ...))
    if (argc != 4 && argc != 5) return 2;
    const bool cols = argc == 5 && argv[4][0] == 'c';
    FILE* f = fopen(argv[1], "rb");
    if (!f) return 3;
    int32_t m = 0, n = 0;
    int64_t nnz = 0;
    bool ok = read_all(f, &m, 4, 1) && read_all(f, &n, 4, 1) && read_all(f, &nnz, 8, 1);
    HostProblem hp;
    hp.m = m;
    hp.n = n;
    hp.ptr.resize(m + 1);
    std::vector<int32_t> idx(nnz);
    std::vector<double> val(nnz, 1.0);
    hp.kind.resize(m);
    std::vector<int32_t> inv_col(n);
    ok = ok && read_all(f, hp.ptr.data(), 4, m + 1) && read_all(f, idx.data(), 4, nnz) &&
         read_all(f, hp.kind.data(), 1, m) && read_all(f, inv_col.data(), 4, n);
    fclose(f);
    if (!ok) return 4;
    // two segments, as the ub and eq parts of a problem arrive
    const int64_t h = nnz / 2;
    hp.segs.push_back({idx.data(), val.data(), h});
    hp.segs.push_back({idx.data() + h, val.data() + h, nnz - h});
    using E = Engine<float>;
    const std::vector<uint8_t> slab = cols ? std::vector<uint8_t>(m, 0) : E::choose_slab(hp, inv_col, 4);
    std::vector<int64_t> rlen(m);
    for (int i = 0; i < m; ++i) rlen[i] = hp.ptr[i + 1] - hp.ptr[i];
    E::Plan P;
    if (cols)
        E::make_plan(rlen, nullptr, nullptr, P, atoi(argv[3]));
    else
        E::make_plan(rlen, &hp.kind, &slab, P, atoi(argv[3]));
    FILE* o = fopen(argv[2], "wb");
    if (!o) return 5;
    auto put = [&](const std::vector<int32_t>& v) {
        const int64_t s = (int64_t)v.size();
        fwrite(&s, 8, 1, o);
        fwrite(v.data(), 4, v.size(), o);
    };
    put(std::vector<int32_t>(slab.begin(), slab.end()));
    put(P.perm);
    put(P.fptr);
    put(P.soff);
    put(P.unit);
    std::vector<int32_t> bins = {P.bt.nbins, P.bt.total_blocks};
    for (int i = 0; i < P.bt.nbins; ++i) {
        const Bin& b = P.bt.bin[i];
        const int32_t v[12] = {b.begin, b.end,   b.mode,  b.kind,   b.block_begin, b.nblocks,
                               b.units, b.aux,   b.aux2,  b.slice0, b.part0,       b.slot0};
        bins.insert(bins.end(), v, v + 12);
    }
    put(bins);
    put({(int32_t)P.total, P.ntickets, P.nslots, P.nslab_units});
    fclose(o);
    return 0;
}
