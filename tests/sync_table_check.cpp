// Host check of the ghost-sync patch tables (make_sync_table,
// wabbit_gb300/csrc/forest.cpp, built from memoised per-relation templates on
// the host thread pool) against a sequential construction from make_patch:
// every sender in order, every relation in ascending order, boxes shifted to
// the buffer's ghost width, patches grouped by stage in that order.
#include "forest.hpp"

#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

using namespace wg;

static int prediction_need(const Patch &p, int order) {
    const int h = order - 1;
    const int cx = p.shi[0] - p.slo[0] + 1, cy = p.shi[1] - p.slo[1] + 1, cz = p.shi[2] - p.slo[2] + 1;
    const int Fy = 2 * cy - 1, Fz = 2 * cz - 1;
    const int ex = p.rhi[0] - p.rlo[0] + 1, ey = p.rhi[1] - p.rlo[1] + 1, ez = p.rhi[2] - p.rlo[2] + 1;
    int yw0 = std::max(0, p.blo[1] - h), yw1 = std::min(Fy - 1, p.blo[1] + ey - 1 + h);
    yw0 += yw0 & 1;
    yw1 -= yw1 & 1;
    int zw0 = std::max(0, p.blo[2] - h), zw1 = std::min(Fz - 1, p.blo[2] + ez - 1 + h);
    zw0 += zw0 & 1;
    zw1 -= zw1 & 1;
    const int wy = (yw1 - yw0) / 2 + 1, wz = (zw1 - zw0) / 2 + 1;
    return cx * cy * cz + ex * wy * wz + ex * ey * wz;
}

int main(int argc, char **argv) {
    if (argc < 2) return 2;
    FILE *fi = std::fopen(argv[1], "r");
    if (!fi) return 2;
    int dim = 0, n = 0;
    if (std::fscanf(fi, "%d %d", &dim, &n) != 2) return 2;
    std::vector<int> lv(n), co(3 * n);
    for (int i = 0; i < n; i++)
        if (std::fscanf(fi, "%d %d %d %d", &lv[i], &co[3 * i], &co[3 * i + 1], &co[3 * i + 2]) != 4) return 2;
    std::fclose(fi);
    Forest f;
    f.dim = dim;
    f.Jmin = 1;
    f.Jmax = 12;
    f.set(n, lv.data(), co.data());
    std::string err;
    if (!f.update_neighbors(err)) {
        std::printf("neighbours: %s\n", err.c_str());
        return 2;
    }
    long cases = 0, bad = 0;
    for (const char *wn : {"CDF40", "CDF44", "CDF22"}) {
        WaveletInfo w;
        make_wavelet(wn, w);
        Geometry geo;
        geo.dim = dim;
        geo.Bs[0] = geo.Bs[1] = 16;
        geo.Bs[2] = dim == 3 ? 16 : 1;
        geo.g = 6;
        geo.nc = dim + 1;
        for (int gm : {2, 4, 6})
            for (int gb : {6, 4}) {
                if (gm > gb) continue;
                cases++;
                SyncTable got;
                if (!make_sync_table(f, geo, w, gm, gm, gb, 3, got, err)) {
                    std::printf("%s gm=%d gbuf=%d: %s\n", wn, gm, gb, err.c_str());
                    bad++;
                    continue;
                }
                const int nst = w.lifted ? 3 : 2, unl = w.lifted ? 0 : 1, sh = geo.g - gb;
                std::vector<std::vector<Patch>> per(nst + 1);
                int max_points = 0, max_coarse = 0;
                for (int s = 0; s < n; s++)
                    for (int r = 1; r <= kNumRelations; r++) {
                        const int d = f.nbr[(size_t)s * kNumRelations + r - 1];
                        if (d < 0) continue;
                        const int ld = f.level[s] - f.level[d];
                        Patch p = make_patch(geo, w.order_predictor, r, ld, gm, gm, s + 3, d + 3);
                        p.stage = (int16_t)(ld == 0 ? 1 : ld == 1 ? 2 - unl : 3 - unl);
                        int npts = 1;
                        for (int k = 0; k < 3; k++) {
                            const int sk = k < dim ? sh : 0;
                            p.rlo[k] -= sk;
                            p.rhi[k] -= sk;
                            p.slo[k] -= sk;
                            p.shi[k] -= sk;
                            npts *= p.rhi[k] - p.rlo[k] + 1;
                        }
                        max_points = std::max(max_points, npts);
                        if (p.op == 2) max_coarse = std::max(max_coarse, prediction_need(p, w.order_predictor));
                        per[p.stage].push_back(p);
                    }
                std::vector<Patch> want;
                std::vector<int> begin(nst + 1, 0);
                for (int st = 1; st <= nst; st++) {
                    begin[st - 1] = (int)want.size();
                    want.insert(want.end(), per[st].begin(), per[st].end());
                }
                begin[nst] = (int)want.size();
                bool same = got.nstages == nst && got.stage_begin == begin && got.max_points == max_points &&
                            got.max_coarse == max_coarse && got.patches.size() == want.size();
                for (size_t i = 0; same && i < want.size(); i++)
                    same = std::memcmp(&got.patches[i], &want[i], sizeof(Patch)) == 0;
                for (int st = 0; same && st < nst; st++) {
                    bool all_pred = begin[st + 1] > begin[st];
                    for (int i = begin[st]; i < begin[st + 1]; i++) all_pred = all_pred && want[i].op == 2;
                    same = got.stage_predict[st] == (all_pred ? 1 : 0);
                }
                if (!same) {
                    std::printf("%s gm=%d gbuf=%d: table differs\n", wn, gm, gb);
                    bad++;
                }
            }
    }
    std::printf("blocks %d tables %ld differing %ld\n", n, cases, bad);
    return bad ? 1 : 0;
}
