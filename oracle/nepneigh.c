/* ORACLE - test infrastructure only, never linked into the product library.
 *
 * CPU restatement of MatPL's NEP neighbor operators:
 *   calculate_neighbor  -> launch_calculate_neighbor_cpu (src/op/src/cpu_calculate_nepneighbor.cpp:105-203)
 *   calculate_maxneigh  -> launch_calculate_maxneigh_cpu (cpu_calculate_nepneighbor.cpp:6-103)
 *   minimum image       -> cpu_dev_apply_mic (src/op/src/nep_cpu.cpp:4-15)
 *
 * For every atom n1 of a frame, candidates run over n2 of the same frame (ascending) and, inside
 * that, over the replica offsets (ia, ib, ic) in [0, num_cell) (ic fastest), skipping n1 itself at
 * offset (0, 0, 0).  The displacement is ((pos2 + delta) - pos1) with delta = box_orig . (ia, ib, ic),
 * folded by the minimum-image convention of the replicated cell (box[9:18] = h^-1, box[0:9] = h),
 * and kept when its squared length is below rc^2.  The floating-point operations are written in
 * the reference's order and this file is compiled with -ffp-contract=off, so the results are the
 * reference's bit for bit.  Unlike the reference (which writes past max_NN unchecked), a list that
 * would overflow stops being written; the count is still complete and the function returns 1.
 */
#include <math.h>
#include <stdint.h>

static void mic(const double *box, double *x12, double *y12, double *z12) {
    double sx = box[9] * *x12 + box[10] * *y12 + box[11] * *z12;
    double sy = box[12] * *x12 + box[13] * *y12 + box[14] * *z12;
    double sz = box[15] * *x12 + box[16] * *y12 + box[17] * *z12;
    sx -= nearbyint(sx);
    sy -= nearbyint(sy);
    sz -= nearbyint(sz);
    *x12 = box[0] * sx + box[1] * sy + box[2] * sz;
    *y12 = box[3] * sx + box[4] * sy + box[5] * sz;
    *z12 = box[6] * sx + box[7] * sy + box[8] * sz;
}

/* displacement of (n2, image) from n1; returns the squared length */
static double disp(const double *pos, const double *bo, const double *box, int64_t n1, int64_t n2,
                   int ia, int ib, int ic, double *x12, double *y12, double *z12) {
    double dx = bo[0] * ia + bo[1] * ib + bo[2] * ic;
    double dy = bo[3] * ia + bo[4] * ib + bo[5] * ic;
    double dz = bo[6] * ia + bo[7] * ib + bo[8] * ic;
    *x12 = pos[n2 * 3] + dx - pos[n1 * 3];
    *y12 = pos[n2 * 3 + 1] + dy - pos[n1 * 3 + 1];
    *z12 = pos[n2 * 3 + 2] + dz - pos[n1 * 3 + 2];
    mic(box, x12, y12, z12);
    return *x12 * *x12 + *y12 * *y12 + *z12 * *z12;
}

/* neighbor lists; NL_* must hold N * max_NN entries (filled with -1 / 0 here), Ri_* N * max_NN * 4
 * (r, x, y, z) when with_rij, else N * max_NN * 3 (x, y, z). */
int oracle_nep_neighbor(int64_t nframes, const int64_t *num_atom, const double *box,
                        const double *box_orig, const int64_t *num_cell, const double *pos,
                        double rc_r, double rc_a, int64_t max_r, int64_t max_a, int with_rij,
                        int64_t *NN_r, int64_t *NL_r, double *Ri_r, int64_t *NN_a, int64_t *NL_a,
                        double *Ri_a) {
    int overflow = 0;
    const int w = with_rij ? 4 : 3;
    int64_t N1 = 0;
    for (int64_t f = 0; f < nframes; ++f) {
        const int64_t N2 = N1 + num_atom[f];
        const double *bx = box + 18 * f, *bo = box_orig + 9 * f;
        const int64_t *nc = num_cell + 3 * f;
        /* centre atoms are independent: with OpenMP they run in parallel (each writes only its
         * own rows, in the serial order) */
#pragma omp parallel for schedule(dynamic, 16) reduction(|| : overflow)
        for (int64_t n1 = N1; n1 < N2; ++n1) {
            for (int64_t s = 0; s < max_r; ++s) NL_r[n1 * max_r + s] = -1;
            for (int64_t s = 0; s < max_a; ++s) NL_a[n1 * max_a + s] = -1;
            for (int64_t s = 0; s < max_r * w; ++s) Ri_r[n1 * max_r * w + s] = 0.0;
            for (int64_t s = 0; s < max_a * w; ++s) Ri_a[n1 * max_a * w + s] = 0.0;
            int64_t cr = 0, ca = 0;
            for (int64_t n2 = N1; n2 < N2; ++n2)
                for (int ia = 0; ia < nc[0]; ++ia)
                    for (int ib = 0; ib < nc[1]; ++ib)
                        for (int ic = 0; ic < nc[2]; ++ic) {
                            if (ia == 0 && ib == 0 && ic == 0 && n1 == n2) continue;
                            double x, y, z;
                            const double d2 = disp(pos, bo, bx, n1, n2, ia, ib, ic, &x, &y, &z);
                            if (d2 < rc_r * rc_r) {
                                if (cr < max_r) {
                                    double *o = Ri_r + (n1 * max_r + cr) * w;
                                    NL_r[n1 * max_r + cr] = n2;
                                    if (with_rij) *o++ = sqrt(d2);
                                    o[0] = x; o[1] = y; o[2] = z;
                                } else {
                                    overflow = 1;
                                }
                                ++cr;
                            }
                            if (d2 < rc_a * rc_a) {
                                if (ca < max_a) {
                                    double *o = Ri_a + (n1 * max_a + ca) * w;
                                    NL_a[n1 * max_a + ca] = n2;
                                    if (with_rij) *o++ = sqrt(d2);
                                    o[0] = x; o[1] = y; o[2] = z;
                                } else {
                                    overflow = 1;
                                }
                                ++ca;
                            }
                        }
            NN_r[n1] = cr;
            NN_a[n1] = ca;
        }
        N1 = N2;
    }
    return overflow;
}

/* neighbor counts only; with_type counts per neighbor element: NN_* [N, ntypes] */
void oracle_nep_maxneigh(int64_t nframes, const int64_t *num_atom, const double *box,
                         const double *box_orig, const int64_t *num_cell, const double *pos,
                         double rc_r, double rc_a, int64_t ntypes, int with_type,
                         const int64_t *type_map, int64_t *NN_r, int64_t *NN_a) {
    int64_t N1 = 0;
    for (int64_t f = 0; f < nframes; ++f) {
        const int64_t N2 = N1 + num_atom[f];
        const double *bx = box + 18 * f, *bo = box_orig + 9 * f;
        const int64_t *nc = num_cell + 3 * f;
#pragma omp parallel for schedule(dynamic, 16)
        for (int64_t n1 = N1; n1 < N2; ++n1) {
            const int64_t nt = with_type ? ntypes : 1;
            for (int64_t t = 0; t < nt; ++t) NN_r[n1 * nt + t] = NN_a[n1 * nt + t] = 0;
            for (int64_t n2 = N1; n2 < N2; ++n2) {
                const int64_t t2 = with_type ? type_map[n2] : 0;
                for (int ia = 0; ia < nc[0]; ++ia)
                    for (int ib = 0; ib < nc[1]; ++ib)
                        for (int ic = 0; ic < nc[2]; ++ic) {
                            if (ia == 0 && ib == 0 && ic == 0 && n1 == n2) continue;
                            double x, y, z;
                            const double d2 = disp(pos, bo, bx, n1, n2, ia, ib, ic, &x, &y, &z);
                            if (d2 < rc_r * rc_r) NN_r[n1 * nt + t2]++;
                            if (d2 < rc_a * rc_a) NN_a[n1 * nt + t2]++;
                        }
            }
        }
        N1 = N2;
    }
}
