/* Random sequential addition of points with a minimum pair separation in a periodic
 * (possibly triclinic) box: the seeded synthetic-structure generator of the benchmark
 * workloads.  Deterministic across machines: integer PRNG (splitmix64) and IEEE double
 * arithmetic compiled without floating-point contraction.
 *
 * Candidates are drawn uniformly in fractional coordinates and rejected when closer
 * than rmin to an accepted point (all periodic images).  A grid of cells whose
 * diagonal is shorter than rmin holds at most one accepted point per cell. */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

static uint64_t next_u64(uint64_t* s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
static double next_unit(uint64_t* s) { return (double)(next_u64(s) >> 11) * (1.0 / 9007199254740992.0); }

static double norm3(const double* v) { return sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]); }
static void cross3(const double* u, const double* v, double* r) {
    r[0] = u[1] * v[2] - u[2] * v[1];
    r[1] = u[2] * v[0] - u[0] * v[2];
    r[2] = u[0] * v[1] - u[1] * v[0];
}

/* box: rows a, b, c.  Writes n x 3 Cartesian positions.  Returns the number placed
 * (n on success; fewer when max_tries candidates in a row were all rejected). */
int rsa_generate(int n, const double* box, double rmin, uint64_t seed, int max_tries, double* out) {
    const double* A = box;
    const double* B = box + 3;
    const double* C = box + 6;
    double bc[3], ca[3], ab[3];
    cross3(B, C, bc);
    cross3(C, A, ca);
    cross3(A, B, ab);
    const double vol = fabs(A[0] * bc[0] + A[1] * bc[1] + A[2] * bc[2]);
    const double h[3] = {vol / norm3(bc), vol / norm3(ca), vol / norm3(ab)};
    const double len[3] = {norm3(A), norm3(B), norm3(C)};
    int nc[3];
    for (int d = 0; d < 3; ++d) nc[d] = (int)floor(len[d] * 1.7320508075688772 * 1.15 / rmin) > 1
                                            ? (int)floor(len[d] * 1.7320508075688772 * 1.15 / rmin) : 1;
    for (;;) {  /* grow the grid until the longest cell diagonal is below rmin */
        double cell[3][3], worst = 0.0;
        for (int d = 0; d < 3; ++d) {
            cell[0][d] = A[d] / nc[0];
            cell[1][d] = B[d] / nc[1];
            cell[2][d] = C[d] / nc[2];
        }
        const int sg[4][3] = {{1, 1, 1}, {1, 1, -1}, {1, -1, 1}, {-1, 1, 1}};
        for (int q = 0; q < 4; ++q) {
            double v[3];
            for (int d = 0; d < 3; ++d) v[d] = sg[q][0] * cell[0][d] + sg[q][1] * cell[1][d] + sg[q][2] * cell[2][d];
            const double l = norm3(v);
            if (l > worst) worst = l;
        }
        if (worst < rmin * 0.999) break;
        for (int d = 0; d < 3; ++d) ++nc[d];
    }
    int R[3];
    for (int d = 0; d < 3; ++d) R[d] = (int)ceil(rmin * nc[d] / h[d]);
    const long long ncell = (long long)nc[0] * nc[1] * nc[2];
    int* grid = (int*)malloc(sizeof(int) * (size_t)ncell);
    double* frac = (double*)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    if (!grid || !frac) { free(grid); free(frac); return -1; }
    for (long long q = 0; q < ncell; ++q) grid[q] = -1;
    uint64_t st = seed;
    const double r2 = rmin * rmin;
    int placed = 0;
    while (placed < n) {
        int ok = 0;
        for (int t = 0; t < max_tries && !ok; ++t) {
            const double s[3] = {next_unit(&st), next_unit(&st), next_unit(&st)};
            int c[3];
            for (int d = 0; d < 3; ++d) {
                c[d] = (int)(s[d] * nc[d]);
                if (c[d] >= nc[d]) c[d] = nc[d] - 1;
            }
            ok = 1;
            for (int oc = -R[2]; oc <= R[2] && ok; ++oc)
                for (int ob = -R[1]; ob <= R[1] && ok; ++ob)
                    for (int oa = -R[0]; oa <= R[0] && ok; ++oa) {
                        const int q[3] = {c[0] + oa, c[1] + ob, c[2] + oc};
                        int img[3], cc[3];
                        for (int d = 0; d < 3; ++d) {
                            img[d] = q[d] >= 0 ? q[d] / nc[d] : -((-q[d] + nc[d] - 1) / nc[d]);
                            cc[d] = q[d] - img[d] * nc[d];
                        }
                        const int o = grid[cc[0] + (long long)nc[0] * (cc[1] + (long long)nc[1] * cc[2])];
                        if (o < 0) continue;
                        const double df[3] = {frac[3 * o] + img[0] - s[0], frac[3 * o + 1] + img[1] - s[1],
                                              frac[3 * o + 2] + img[2] - s[2]};
                        double d2 = 0.0;
                        for (int d = 0; d < 3; ++d) {
                            const double v = df[0] * A[d] + df[1] * B[d] + df[2] * C[d];
                            d2 += v * v;
                        }
                        if (d2 < r2) ok = 0;
                    }
            if (ok) {
                for (int d = 0; d < 3; ++d) frac[3 * placed + d] = s[d];
                grid[c[0] + (long long)nc[0] * (c[1] + (long long)nc[1] * c[2])] = placed;
            }
        }
        if (!ok) break;
        ++placed;
    }
    for (int i = 0; i < placed; ++i)
        for (int d = 0; d < 3; ++d)
            out[3 * i + d] = frac[3 * i] * A[d] + frac[3 * i + 1] * B[d] + frac[3 * i + 2] * C[d];
    free(grid);
    free(frac);
    return placed;
}
