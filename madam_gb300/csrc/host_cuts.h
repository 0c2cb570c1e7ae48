// host_cuts.h -- host-side cut encoding and the per-call sparse structures
// (B^T incidence in cut order, B B^T + I in CSR) uploaded for the ADMM.
#pragma once
#include <algorithm>
#include <cstdint>
#include <vector>

#include "mcb_dev.cuh"

namespace mcb {

struct CutLists {
    std::vector<int> tri, pent, hept;  // reference layouts: 4 / 6 / 8 ints per cut
    int m() const { return (int)(tri.size() / 4 + pent.size() / 6 + hept.size() / 8); }
};

// --- cut encoding ----------------------------------------------------------
// tri (i,j,k,type): signs of op_B (operators.c:81-96); pent / hept: H = e e^T with
// e_a = -1 for a < type-1 (cutting_planes.c:242-244, 438-441).
inline void encode_cut(int k, const int *c, int *cp) {
    int sign = 0;
    if (k == 3) {
        static const int sm[4] = {0, 4, 2, 1};  // type 1..4 -> mask of negative e_a
        int type = c[3];
        sign = sm[(type >= 1 && type <= 4) ? type - 1 : 3];
        cp[1] = c[0];
        cp[2] = c[1];
        cp[3] = c[2];
    } else {
        int type = c[0];
        for (int a = 0; a < type - 1 && a < 3; ++a) sign |= 1 << a;
        for (int a = 0; a < k; ++a) cp[1 + a] = c[1 + a];
    }
    cp[0] = k | (sign << 8);
    for (int a = k; a < 7; ++a) cp[1 + a] = 0;
}

struct HostCuts {
    std::vector<int> cp;                           // 8 per cut
    std::vector<int> e_idx, e_rp, e_cut;           // B^T incidence
    std::vector<double> e_coef;
    std::vector<int> g_rp, g_ci;                   // B B^T + I
    std::vector<double> g_v;
};

inline void build_host_cuts(const CutLists &r, int n, HostCuts &H) {

    const int m = r.m();
    H.cp.assign((size_t)8 * m, 0);
    int q = 0;
    for (size_t a = 0; a < r.tri.size() / 4; ++a, ++q) encode_cut(3, &r.tri[4 * a], &H.cp[8 * (size_t)q]);
    for (size_t a = 0; a < r.pent.size() / 6; ++a, ++q) encode_cut(5, &r.pent[6 * a], &H.cp[8 * (size_t)q]);
    for (size_t a = 0; a < r.hept.size() / 8; ++a, ++q) encode_cut(7, &r.hept[8 * a], &H.cp[8 * (size_t)q]);
    // incidence triples (edge, cut, coef) in cut order
    struct Inc { int edge, cut; double coef; };
    std::vector<Inc> inc;
    inc.reserve((size_t)21 * m);
    for (int c = 0; c < m; ++c) {
        const int *cp = &H.cp[8 * (size_t)c];
        int h = cp[0], k = cut_k(h);
        double half = 0.5 * cut_scale(k);
        for (int a = 0; a < k; ++a)
            for (int b = a + 1; b < k; ++b) {
                int i = cp[1 + a], j = cp[1 + b];
                int lo = i < j ? i : j, hi = i < j ? j : i;
                double coef = (cut_sign(h, a) * cut_sign(h, b) > 0) ? half : -half;
                inc.push_back({hi + lo * n, c, coef});
            }
    }
    std::stable_sort(inc.begin(), inc.end(), [](const Inc &x, const Inc &y) { return x.edge < y.edge; });
    H.e_idx.clear();
    H.e_rp.clear();
    H.e_cut.resize(inc.size());
    H.e_coef.resize(inc.size());
    for (size_t a = 0; a < inc.size(); ++a) {
        if (a == 0 || inc[a].edge != inc[a - 1].edge) {
            H.e_idx.push_back(inc[a].edge);
            H.e_rp.push_back((int)a);
        }
        H.e_cut[a] = inc[a].cut;
        H.e_coef[a] = inc[a].coef;
    }
    H.e_rp.push_back((int)inc.size());
    // G = B B^T + I, entries 2 * sum over shared edges of coef_a coef_b
    std::vector<std::pair<uint64_t, double>> tr;
    tr.reserve((size_t)m + inc.size() * 4);
    for (int c = 0; c < m; ++c) tr.push_back({(uint64_t)c * m + c, 1.0});
    for (size_t e = 0; e + 1 < H.e_rp.size(); ++e)
        for (int a = H.e_rp[e]; a < H.e_rp[e + 1]; ++a)
            for (int b = H.e_rp[e]; b < H.e_rp[e + 1]; ++b)
                tr.push_back({(uint64_t)H.e_cut[a] * m + H.e_cut[b], 2.0 * H.e_coef[a] * H.e_coef[b]});
    std::stable_sort(tr.begin(), tr.end(),
                     [](const std::pair<uint64_t, double> &x, const std::pair<uint64_t, double> &y) {
                         return x.first < y.first;
                     });
    H.g_rp.assign((size_t)m + 1, 0);
    H.g_ci.clear();
    H.g_v.clear();
    for (size_t a = 0; a < tr.size();) {
        size_t b = a;
        double acc = 0.0;
        while (b < tr.size() && tr[b].first == tr[a].first) acc += tr[b++].second;
        int row = (int)(tr[a].first / m), col = (int)(tr[a].first % m);
        H.g_ci.push_back(col);
        H.g_v.push_back(acc);
        H.g_rp[row + 1]++;
        a = b;
    }
    for (int r2 = 0; r2 < m; ++r2) H.g_rp[r2 + 1] += H.g_rp[r2];
}


}  // namespace mcb
