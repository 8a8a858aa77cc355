// Coefficient tables of the three- and four-body invariant columns, generated from the
// Wigner 3j and Clebsch-Gordan definitions in invariants.hpp.  The 3j symbols use
// Racah's closed form with long-double factorials (exact up to 20!, enough for l <= 6).
#include "invariants.hpp"

#include <algorithm>
#include <array>
#include <cmath>
#include <complex>
#include <map>
#include <stdexcept>

namespace nnapgb {
namespace {

using cplx = std::complex<double>;

const int kL3[][3] = {{2, 2, 2}, {1, 1, 2}, {2, 3, 3}, {1, 2, 3}, {4, 4, 4}, {2, 2, 4}, {3, 3, 4}, {2, 4, 4},
                      {1, 3, 4}, {2, 5, 5}, {4, 5, 5}, {2, 3, 5}, {1, 4, 5}, {3, 4, 5}, {6, 6, 6}, {3, 3, 6},
                      {4, 4, 6}, {5, 5, 6}, {2, 6, 6}, {4, 6, 6}, {2, 4, 6}, {1, 5, 6}, {3, 5, 6}};
const int kL3Cols[7] = {0, 0, 2, 4, 9, 14, 23};  // columns for l3max = 0..6
const int kL4[][4] = {{1, 1, 1, 1}, {2, 2, 2, 2}, {1, 1, 2, 2}, {3, 3, 3, 3}, {1, 1, 3, 3},
                      {2, 2, 3, 3}, {1, 1, 1, 3}, {1, 3, 3, 3}, {1, 2, 2, 3}};
const int kL4Cols[4] = {0, 1, 3, 9};             // columns for l4max = 0..3

long double fact(int n) {
    long double f = 1.0L;
    for (int i = 2; i <= n; ++i) f *= i;
    return f;
}

double wigner3j(int j1, int j2, int j3, int m1, int m2, int m3) {
    if (m1 + m2 + m3 != 0 || j3 < std::abs(j1 - j2) || j3 > j1 + j2) return 0.0;
    if (std::abs(m1) > j1 || std::abs(m2) > j2 || std::abs(m3) > j3) return 0.0;
    const long double tri = fact(j1 + j2 - j3) * fact(j1 - j2 + j3) * fact(-j1 + j2 + j3) / fact(j1 + j2 + j3 + 1);
    const long double pre = tri * fact(j1 + m1) * fact(j1 - m1) * fact(j2 + m2) * fact(j2 - m2) * fact(j3 + m3) *
                            fact(j3 - m3);
    long double s = 0.0L;
    for (int k = 0; k <= j1 + j2 + j3; ++k) {
        const int d[6] = {k, j3 - j2 + k + m1, j3 - j1 + k - m2, j1 + j2 - j3 - k, j1 - k - m1, j2 - k + m2};
        if (*std::min_element(d, d + 6) < 0) continue;
        long double den = 1.0L;
        for (int x : d) den *= fact(x);
        s += ((k & 1) ? -1.0L : 1.0L) / den;
    }
    const int e = j1 - j2 - m3;
    const long double sign = (((e % 2) + 2) % 2) ? -1.0L : 1.0L;
    return (double)(sign * s * std::sqrt(pre));
}

double clebsch(int j1, int m1, int j2, int m2, int J, int M) {
    const int e = j1 - j2 + M;
    const double sign = (((e % 2) + 2) % 2) ? -1.0 : 1.0;
    return sign * std::sqrt(2.0 * J + 1.0) * wigner3j(j1, j2, J, m1, m2, -M);
}

// a_{l mu} = sum over (m, v) of v A_{l m}
struct VEntry {
    int m;
    cplx v;
};
std::vector<VEntry> vrow(int mu) {
    const double r2 = 1.0 / std::sqrt(2.0);
    if (mu == 0) return {{0, cplx(1.0, 0.0)}};
    const int m = std::abs(mu);
    const double s = (m & 1) ? -1.0 : 1.0;
    if (mu > 0) return {{m, cplx(s * r2, 0.0)}, {-m, cplx(0.0, s * r2)}};
    return {{m, cplx(r2, 0.0)}, {-m, cplx(0.0, -r2)}};
}

int lm(int l, int m) { return l * l + l + m; }

using Key = std::array<int, 4>;

std::vector<InvTerm> fold(const std::map<Key, cplx>& acc, int order) {
    std::map<Key, double> out;
    for (auto& kv : acc) {
        Key k = kv.first;
        std::sort(k.begin(), k.begin() + order);
        out[k] += kv.second.real();
    }
    std::vector<InvTerm> t;
    for (auto& kv : out) {
        if (std::fabs(kv.second) <= 1e-13) continue;
        InvTerm x;
        x.order = order;
        for (int q = 0; q < 4; ++q) x.idx[q] = q < order ? kv.first[q] : -1;
        x.coeff = kv.second;
        t.push_back(x);
    }
    return t;
}

std::vector<InvTerm> l3_terms(int l1, int l2, int l3) {
    std::map<Key, cplx> acc;
    for (int u1 = -l1; u1 <= l1; ++u1)
        for (int u2 = -l2; u2 <= l2; ++u2) {
            const int u3 = -u1 - u2;
            if (std::abs(u3) > l3) continue;
            const double w = wigner3j(l1, l2, l3, u1, u2, u3);
            if (w == 0.0) continue;
            for (auto& a : vrow(u1))
                for (auto& b : vrow(u2))
                    for (auto& c : vrow(u3)) acc[Key{lm(l1, a.m), lm(l2, b.m), lm(l3, c.m), -1}] += w * a.v * b.v * c.v;
        }
    return fold(acc, 3);
}

std::vector<InvTerm> l4_terms(int l1, int l2, int l3, int l4) {
    std::map<Key, cplx> acc;
    for (int L = std::abs(l1 - l2); L <= l1 + l2; ++L) {
        if (L < std::abs(l3 - l4) || L > l3 + l4) continue;
        const double wL = (((l1 + l2 + L) & 1) ? -1.0 : 1.0) / (2.0 * L + 1.0);
        for (int M = -L; M <= L; ++M) {
            std::map<std::pair<int, int>, cplx> left, right;
            for (int u1 = -l1; u1 <= l1; ++u1) {
                const int u2 = M - u1;
                if (std::abs(u2) > l2) continue;
                const double c = clebsch(l1, u1, l2, u2, L, M);
                if (c == 0.0) continue;
                for (auto& a : vrow(u1))
                    for (auto& b : vrow(u2)) left[{lm(l1, a.m), lm(l2, b.m)}] += c * a.v * b.v;
            }
            for (int u3 = -l3; u3 <= l3; ++u3) {
                const int u4 = M - u3;
                if (std::abs(u4) > l4) continue;
                const double c = clebsch(l3, u3, l4, u4, L, M);
                if (c == 0.0) continue;
                for (auto& a : vrow(u3))
                    for (auto& b : vrow(u4)) right[{lm(l3, a.m), lm(l4, b.m)}] += c * std::conj(a.v * b.v);
            }
            for (auto& x : left)
                for (auto& y : right)
                    acc[Key{x.first.first, x.first.second, y.first.first, y.first.second}] += wL * x.second * y.second;
        }
    }
    return fold(acc, 4);
}

}  // namespace

int invariant_count(int l3max, int l4max) {
    if (l3max < 0 || l3max > 6 || l4max < 0 || l4max > 3) throw std::runtime_error("l3max/l4max out of range");
    return kL3Cols[l3max] + kL4Cols[l4max];
}

std::vector<std::vector<InvTerm>> invariant_columns(int l3max, int l4max) {
    invariant_count(l3max, l4max);
    std::vector<std::vector<InvTerm>> cols;
    for (int c = 0; c < kL3Cols[l3max]; ++c) cols.push_back(l3_terms(kL3[c][0], kL3[c][1], kL3[c][2]));
    for (int c = 0; c < kL4Cols[l4max]; ++c) cols.push_back(l4_terms(kL4[c][0], kL4[c][1], kL4[c][2], kL4[c][3]));
    return cols;
}

}  // namespace nnapgb
