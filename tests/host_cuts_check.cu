// Host-only check of madam_gb300/csrc/host_cuts.h (no kernel is launched): reads
// cut lists, a matrix X and a dual vector t on stdin, and writes what the library
// uploads for one ADMM call, in terms a test can compare with the oracle:
//   y   = B(X) through the packed cut encoding (scale * sum_{a<b} -e_a e_b X_ab, X read
//         through its lower triangle),
//   Z   = sum_c t_c A_c scattered through the edge incidence (both triangles),
//   G   = B B^T + I from the CSR, as a dense m x m matrix (row-major).
// Input (whitespace separated): n, ntri, 4*ntri ints, npent, 6*npent ints,
// nhept, 8*nhept ints, n*n doubles of X (column-major), m doubles of t.
// Output: m doubles of y, n*n doubles of Z, m*m doubles of G, one per line (%.17g).
#include <cstdio>
#include <vector>

#include "../madam_gb300/csrc/host_cuts.h"

using namespace mcb;

static bool read_ints(std::vector<int> &v, int count) {
    v.resize(count);
    for (int &x : v)
        if (std::scanf("%d", &x) != 1) return false;
    return true;
}

int main() {
    int n, nt, np, nh;
    CutLists cl;
    if (std::scanf("%d %d", &n, &nt) != 2 || !read_ints(cl.tri, 4 * nt)) return 2;
    if (std::scanf("%d", &np) != 1 || !read_ints(cl.pent, 6 * np)) return 2;
    if (std::scanf("%d", &nh) != 1 || !read_ints(cl.hept, 8 * nh)) return 2;
    const int m = cl.m();
    std::vector<double> X((size_t)n * n), t(m);
    for (double &x : X)
        if (std::scanf("%lf", &x) != 1) return 2;
    for (double &x : t)
        if (std::scanf("%lf", &x) != 1) return 2;
    HostCuts H;
    build_host_cuts(cl, n, H);
    for (int c = 0; c < m; ++c) {
        const int *cp = &H.cp[8 * (size_t)c];
        const int h = cp[0], k = cut_k(h);
        double acc = 0.0;
        for (int a = 0; a < k; ++a)
            for (int b = a + 1; b < k; ++b) {
                int i = cp[1 + a], j = cp[1 + b];
                int lo = i < j ? i : j, hi = i < j ? j : i;
                acc += -(double)(cut_sign(h, a) * cut_sign(h, b)) * X[hi + (size_t)lo * n];
            }
        std::printf("%.17g\n", cut_scale(k) * acc);
    }
    std::vector<double> Z((size_t)n * n, 0.0);
    for (size_t e = 0; e + 1 < H.e_rp.size(); ++e) {
        const int idx = H.e_idx[e], hi = idx % n, lo = idx / n;
        for (int a = H.e_rp[e]; a < H.e_rp[e + 1]; ++a) {
            const double v = H.e_coef[a] * t[H.e_cut[a]];
            Z[hi + (size_t)lo * n] += v;
            Z[lo + (size_t)hi * n] += v;
        }
    }
    for (double z : Z) std::printf("%.17g\n", z);
    std::vector<double> G((size_t)m * m, 0.0);
    for (int r = 0; r < m; ++r)
        for (int a = H.g_rp[r]; a < H.g_rp[r + 1]; ++a) G[(size_t)r * m + H.g_ci[a]] = H.g_v[a];
    for (double g : G) std::printf("%.17g\n", g);
    return 0;
}
