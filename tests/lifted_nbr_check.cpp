// Host check of the full-tree neighbour lists of the lifted adaptation
// (LiftedTree::update_metadata, wabbit_gb300/csrc/lifted.cpp): for several
// alive sets, the lists must equal a direct restatement of find_neighbor
// with search_overlapping (LIB/MESH/find_neighbors.f90:18-215) restricted to
// alive blocks: the same-level block, the finer parts up to the first one
// that is missing or not alive, and the coarser block when this block touches
// its mother's boundary in that direction.
#include "lifted.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <utility>
#include <vector>

using namespace wg;

static std::vector<std::pair<int, int>> direct(const LiftedTree &L, int b) {
    std::vector<std::pair<int, int>> out;
    const FullTree &ft = L.ft;
    const int dim = ft.dim, lv = ft.level[b], N = 1 << lv;
    const int *c = &ft.coords[3 * b];
    for (int dz = (dim == 3 ? -1 : 0); dz <= (dim == 3 ? 1 : 0); dz++)
        for (int dy = -1; dy <= 1; dy++)
            for (int dx = -1; dx <= 1; dx++) {
                if (!dx && !dy && !dz) continue;
                const int d[3] = {dx, dy, dz};
                int nfree = 0;
                for (int i = 0; i < dim; i++) nfree += (d[i] == 0);
                int a[3] = {0, 0, 0};
                for (int i = 0; i < dim; i++) a[i] = ((c[i] + d[i]) % N + N) % N;
                const int same = lv == 0 ? b : ft.find(lv, a[0], a[1], a[2]);
                if (same >= 0 && L.alive[same]) out.push_back({relation_id(d, 0, dim), same});
                if (lv < L.Jmax && same >= 0)
                    for (int p = 0; p < (1 << nfree); p++) {
                        int k = 0, fr = 0;
                        for (int i = 0; i < dim; i++) {
                            const int bit = d[i] == 0 ? (p >> fr++) & 1 : (d[i] > 0 ? 1 : 0);
                            k |= (((bit + d[i]) % 2 + 2) % 2) << i;
                        }
                        const int f = ft.daughters[8 * same + k];
                        if (f < 0 || !L.alive[f]) break;
                        out.push_back({relation_id(d, p, dim) + 112, f});
                    }
                if (lv <= L.Jmin) continue;
                int prt = 0, fr = 0;
                bool touches = true;
                for (int i = 0; i < dim; i++) {
                    const int bit = c[i] & 1;
                    if (d[i] == 0) prt |= bit << fr++;
                    else if ((d[i] > 0) != (bit == 1)) touches = false;
                }
                if (!touches) continue;
                const int cb = same >= 0 ? ft.mother[same] : ft.find(lv - 1, a[0] >> 1, a[1] >> 1, a[2] >> 1);
                if (cb >= 0 && L.alive[cb]) out.push_back({relation_id(d, prt, dim) + 56, cb});
            }
    std::sort(out.begin(), out.end());
    return out;
}

int main(int argc, char **argv) {
    if (argc < 4) return 2;
    FILE *fi = std::fopen(argv[1], "r");
    if (!fi) return 2;
    int dim = 0, n = 0;
    if (std::fscanf(fi, "%d %d", &dim, &n) != 2) return 2;
    std::vector<int> lv(n), co(3 * n);
    for (int i = 0; i < n; i++)
        if (std::fscanf(fi, "%d %d %d %d", &lv[i], &co[3 * i], &co[3 * i + 1], &co[3 * i + 2]) != 4) return 2;
    std::fclose(fi);
    Geometry geo;
    geo.dim = dim;
    geo.Bs[0] = geo.Bs[1] = 16;
    geo.Bs[2] = dim == 3 ? 16 : 1;
    geo.g = 6;
    geo.nc = dim + 1;
    WaveletInfo w;
    make_wavelet("CDF44", w);
    LiftedTree L;
    std::string err;
    if (!L.init(geo, w, 2, std::atoi(argv[2]), std::atoi(argv[3]), n, lv.data(), co.data(), err)) {
        std::printf("init failed: %s\n", err.c_str());
        return 2;
    }
    unsigned long long rng = 0x2545F4914F6CDD1DULL;
    auto rnd = [&]() {
        rng ^= rng << 13;
        rng ^= rng >> 7;
        rng ^= rng << 17;
        return (unsigned)(rng % 100);
    };
    long mismatches = 0, lists = 0;
    for (int pattern = 0; pattern < 6; pattern++) {
        for (int b = 0; b < L.size(); b++)
            L.alive[b] = pattern == 0 ? b < n : pattern == 1 ? 1 : rnd() < 60u + 8u * pattern;
        L.update_metadata(err);
        for (int b = 0; b < L.size(); b++) {
            std::vector<std::pair<int, int>> got;
            if (L.alive[b]) L.for_neighbors(b, [&](int r, int nb) { got.push_back({r, nb}); });
            const std::vector<std::pair<int, int>> want =
                L.alive[b] ? direct(L, b) : std::vector<std::pair<int, int>>();
            lists++;
            if (got != want) mismatches++;
        }
    }
    std::printf("blocks %d lists %ld neighbour mismatches %ld\n", L.size(), lists, mismatches);
    return mismatches ? 1 : 0;
}
