// Invariants of the aggregate partition over the PCG blocks (csrc/agg_rounds.h)
// on seeded aggregate layouts: dense aggregates of 1..32 vertices (m x m inverse
// entries) mixed with packs of isolated vertices (9 entries per vertex), grids from
// 1 block to more blocks than aggregates, the FP32 and FP64 staging limits.
// Prints one line per failed check and exits non-zero on any failure.
#include <cstdio>
#include <random>
#include <vector>

#include "../../codim-ipc_gb300/csrc/agg_rounds.h"

static int fails = 0;
#define CHECK(c, ...)                          \
    do {                                       \
        if (!(c)) {                            \
            std::printf("FAIL " __VA_ARGS__);  \
            std::printf("\n");                 \
            ++fails;                           \
        }                                      \
    } while (0)

int main()
{
    std::mt19937 rng(7);
    int layouts = 0;
    for (int trial = 0; trial < 60; ++trial) {
        const int nagg = trial % 10 == 0 ? 1 + (int)(rng() % 3) : 1 + (int)(rng() % 3000);
        const double pack_frac = (trial % 3) * 0.25;
        std::vector<int> voff(1, 0);
        std::vector<long long> boff(1, 0);
        for (int a = 0; a < nagg; ++a) {
            const bool pk = std::uniform_real_distribution<double>(0, 1)(rng) < pack_frac;
            const int sv = pk ? 2 + (int)(rng() % 31) : 1 + (int)(rng() % 32);
            voff.push_back(voff.back() + sv);
            boff.push_back(boff.back() + (pk ? 9LL * sv : 9LL * sv * sv));
        }
        for (int grid : {1, 7, 152, 304, 4000}) {
            for (int rows : {384, 768}) {
                for (int loads : {18, 48}) {
                    const int maxagg = 64;
                    std::vector<int> br, rs;
                    cipc::agg_partition(voff, boff, grid, rows, maxagg, loads, br, rs);
                    ++layouts;
                    const int R = (int)rs.size() - 1;
                    CHECK((int)br.size() == grid + 1, "bround size %d grid %d", (int)br.size(), grid);
                    CHECK(br[0] == 0 && br[grid] == R, "bround ends %d %d rounds %d", br[0], br[grid], R);
                    for (int b = 0; b < grid; ++b) CHECK(br[b] <= br[b + 1], "bround not monotone at %d", b);
                    CHECK(rs.front() == 0 && rs.back() == nagg, "rstart ends %d %d nagg %d", rs.front(), rs.back(),
                          nagg);
                    // rounds: non-empty, within the limits (so every aggregate is in
                    // exactly one round: strictly increasing starts from 0 to nagg)
                    for (int q = 0; q < R; ++q) {
                        CHECK(rs[q] < rs[q + 1], "empty round %d", q);
                        const int nr = 3 * (voff[rs[q + 1]] - voff[rs[q]]);
                        CHECK(nr <= rows, "round %d has %d rows > %d", q, nr, rows);
                        CHECK(rs[q + 1] - rs[q] <= maxagg, "round %d has %d aggregates", q, rs[q + 1] - rs[q]);
                    }
                    // balance: a block's cost exceeds the mean by less than one aggregate
                    std::vector<long long> cost(nagg + 1, 0);
                    long long cmax = 0;
                    for (int g = 0; g < nagg; ++g) {
                        const int sv = voff[g + 1] - voff[g], m = 3 * sv;
                        const bool pk = sv > 1 && boff[g + 1] - boff[g] == 9LL * sv;
                        const long long c = 128LL * cipc::agg_items(m, pk, loads) + 10LL * m;
                        cost[g + 1] = cost[g] + c;
                        cmax = c > cmax ? c : cmax;
                    }
                    const double mean = (double)cost[nagg] / grid;
                    for (int b = 0; b < grid; ++b) {
                        const long long cb = cost[rs[br[b + 1]]] - cost[rs[br[b]]];
                        CHECK(cb <= mean + cmax + 1, "block %d cost %lld mean %.1f max aggregate %lld", b, cb, mean,
                              cmax);
                    }
                    // the kernel's shared slots hold every item of an aggregate of up
                    // to 96 rows (8 at 48 loads, 16 at 18)
                    for (int m = 3; m <= 96; m += 3) {
                        const int it = cipc::agg_items(m, false, loads);
                        CHECK(it <= (loads == 48 ? 8 : 16), "m %d loads %d items %d", m, loads, it);
                        CHECK(it * cipc::agg_cols(m, loads) >= m, "m %d items do not cover the columns", m);
                    }
                }
            }
        }
    }
    std::printf("layouts %d failures %d\n", layouts, fails);
    return fails ? 1 : 0;
}
