// Host partition of the aggregates over the PCG kernel's blocks (aggregate block
// Jacobi, sim_aggregate.cu / sim_pcg.cu).  Plain C++ apart from the item count,
// which the kernel shares: the library builds the tables with it, and a host test
// checks its invariants.
#pragma once
#include <vector>

#ifdef __CUDACC__
#define CIPC_AGG_HD __host__ __device__
#else
#define CIPC_AGG_HD
#endif

namespace cipc {

// Items of the solver's dense aggregate products: an aggregate of m rows takes
// ceil(m / C) items of C = loads / ceil(m / 32) columns (agg_cols; none for a
// pack of isolated vertices, which keeps only 3x3 blocks).
CIPC_AGG_HD inline int agg_cols(int m, int loads)
{
    const int C = loads / ((m + 31) / 32);
    return C > 1 ? C : 1;
}
CIPC_AGG_HD inline int agg_items(int m, bool packed, int loads)
{
    if (packed) return 0;
    const int C = agg_cols(m, loads);
    return (m + C - 1) / C;
}

// voff[a] / boff[a]: vertex and inverse-entry offsets of aggregate a (nagg + 1
// entries each; a pack of isolated vertices holds 9 entries per vertex).  Block
// b of `grid` owns the aggregates whose cost prefix lies in [T b / grid,
// T (b + 1) / grid): T the total cost, the phase waits on an L2 round trip per
// item of a warp (8 warps: 128 per item in units of 1/1024) and per two rows of a
// thread (256 threads: 10 per scalar row).  Each block's range is cut greedily
// into rounds of at most `rows` scalar rows and `maxagg` aggregates.  Output:
// bround (grid + 1 entries) = the first round of each block, rstart (rounds + 1)
// = the first aggregate of each round, rstart.back() = nagg.  Requires every
// aggregate to have at most `rows` rows.
inline void agg_partition(const std::vector<int>& voff, const std::vector<long long>& boff, int grid, int rows,
                          int maxagg, int loads, std::vector<int>& bround, std::vector<int>& rstart)
{
    const int nagg = (int)voff.size() - 1;
    std::vector<long long> cost(nagg + 1, 0);
    for (int g = 0; g < nagg; ++g) {
        const int sv = voff[g + 1] - voff[g], m = 3 * sv;
        const bool pk = sv > 1 && boff[g + 1] - boff[g] == 9LL * sv;
        cost[g + 1] = cost[g] + 128LL * agg_items(m, pk, loads) + 10LL * m;
    }
    const long long T = cost[nagg];
    bround.assign(grid + 1, 0);
    rstart.clear();
    rstart.reserve(nagg + 1);
    int a = 0;
    for (int b = 0; b < grid; ++b) {
        bround[b] = (int)rstart.size();
        const long long end = T * (b + 1) / grid;
        int hi = a;
        while (hi < nagg && (b + 1 == grid || cost[hi] < end)) ++hi;
        for (int g = a; g < hi;) {
            rstart.push_back(g);
            int nr = 0, cnt = 0;
            while (g < hi && cnt < maxagg && nr + 3 * (voff[g + 1] - voff[g]) <= rows) {
                nr += 3 * (voff[g + 1] - voff[g]);
                ++cnt;
                ++g;
            }
        }
        a = hi;
    }
    bround[grid] = (int)rstart.size();
    rstart.push_back(nagg);
}

}  // namespace cipc
