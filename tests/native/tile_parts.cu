// Host check of the tile partitions behind the two-stream launches: the
// near and far parts of a block step's panel tiles (spk::panel_tile) and of
// a front's tensor-core Schur tiles (spk::schur_part_count / _tile) cover
// every tile of the one-launch form exactly once, and a Schur tile is near
// exactly when it holds an entry whose target is factored at the next level
// (a row or column tile below q).  Prints "cases N bad 0" on success.
#include <cstdio>
#include <vector>

#include "spk_kernels.cuh"

using namespace spk;

static int check_panels(int& cases) {
    int bad = 0;
    for (int sym = 0; sym < 2; ++sym)
        for (int nf = 1; nf < 700; nf += 7)
            for (int m = 0; m < 500; m += 13)
                for (int c1 = nf < 128 ? nf : 128; c1 <= nf; c1 += 64) {
                    const int ld = nf + m, nL = cdiv(ld - c1, 64), nUa = cdiv(nf - c1, 64), nU12 = cdiv(m, 64);
                    const int tp = nL + (sym ? 0 : nUa + nU12);
                    if (tp <= 0) continue;
                    ++cases;
                    const int tn = (nL < 2 ? nL : 2) + (sym ? 0 : (nUa < 2 ? nUa : 2));
                    std::vector<int> seen(tp, 0);
                    for (int part = 1; part <= 2; ++part)
                        for (int t = 0; t < (part == 1 ? tn : tp - tn); ++t) {
                            const int u = panel_tile(part, t, nL, nUa, sym != 0);
                            if (u < 0 || u >= tp) { ++bad; continue; }
                            ++seen[u];
                            // near: the first two line tiles of each side
                            const bool isnear = u < nL ? u < 2 : (u - nL < nUa && u - nL < 2);
                            if (isnear != (part == 1)) ++bad;
                        }
                    for (int u = 0; u < tp; ++u) bad += seen[u] != 1;
                }
    return bad;
}

static int check_schur(int& cases) {
    int bad = 0;
    for (int sym = 0; sym < 2; ++sym)
        for (int nh = 1; nh <= 2; ++nh)
            for (int n2 = 1; n2 <= 40; ++n2)
                for (int q = 0; q <= n2 + 2; ++q) {
                    ++cases;
                    const int all = schur_part_count(0, n2, nh, q, sym != 0);
                    const int nn = schur_part_count(1, n2, nh, q, sym != 0), nf = schur_part_count(2, n2, nh, q, sym != 0);
                    if (nn + nf != all) { ++bad; continue; }
                    std::vector<int> seen(all, 0);
                    for (int part = 1; part <= 2; ++part)
                        for (int e = 0; e < (part == 1 ? nn : nf); ++e) {
                            const int t = schur_part_tile(part, e, n2, nh, q, sym != 0);
                            if (t < 0 || t >= all) { ++bad; continue; }
                            ++seen[t];
                            int rt, g;
                            if (sym) lower_tile_w(t, n2, nh, rt, g);
                            else { rt = t % n2; g = t / n2; }
                            const bool isnear = rt < q || nh * g < q;
                            if (isnear != (part == 1)) ++bad;
                        }
                    for (int t = 0; t < all; ++t) bad += seen[t] != 1;
                }
    return bad;
}

int main() {
    int cases = 0;
    const int bad = check_panels(cases) + check_schur(cases);
    std::printf("cases %d bad %d\n", cases, bad);
    return bad != 0;
}
