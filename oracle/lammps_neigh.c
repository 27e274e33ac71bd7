/* ORACLE (test infrastructure only): CPU restatement of PairMATPL::generate_neighdata,
 * src/lmps/lammps-libtorch/MATPL/pair_matpl.cpp:522-616, for checking the GPU conversion of a
 * LAMMPS full neighbor list into per-type DP slots.  Only tests, the package's smoke check and
 * the benchmark's CPU-baseline leg use it.
 *
 * Inputs follow LAMMPS: ilist [inum], the list of row ii is jflat[jstart[ii] .. jstart[ii+1])
 * (LAMMPS firstneigh[ilist[ii]] / numneigh[ilist[ii]] packed in row order), x [nall][3],
 * type [nall] 1-based, type_to_model [ntypes_lmp] (model_atom_type_idx, pair_matpl.cpp:293).
 * Outputs: list_neigh [inum][nt*m] (j+1, 0 empty), dR [inum][nt*m][4] (r, dx, dy, dz),
 * type_map [inum], *min_rsq (starts at 1000 like min_dR, pair_matpl.cpp:539).
 * Returns 1 when a type block would hold more than m neighbors (the reference then writes
 * past the block; here the extra neighbors are counted but not stored), else 0.
 * Built with -ffp-contract=off: rsq = delx*delx + dely*dely + delz*delz in source order.
 */
#include <math.h>
#include <stdlib.h>
#include <string.h>

int oracle_lammps_dp_neighdata(int inum, const int *ilist, const long long *jstart,
                               const int *jflat, const double *x, const int *type,
                               const int *type_to_model, int nt, int m, double cutoff,
                               int *list_neigh, double *dR, int *type_map, double *min_rsq) {
    const double rc2 = cutoff * cutoff;          /* :536 */
    double min_dR = 1000;                        /* :539 */
    int overflow = 0;
    int *num_neigh = (int *)calloc((size_t)nt, sizeof(int));
    const long long S = (long long)nt * m;
    /* vectors are fresh every call (zero-filled by resize on an empty vector, :550-552) */
    memset(list_neigh, 0, sizeof(int) * (size_t)inum * (size_t)S);
    memset(dR, 0, sizeof(double) * 4 * (size_t)inum * (size_t)S);
    for (int ii = 0; ii < inum; ii++) {                                   /* :571 */
        const int i = ilist[ii];
        const int itype = type_to_model[type[i] - 1] + 1;                 /* :559, :574 */
        type_map[ii] = itype - 1;                                         /* :577 */
        memset(num_neigh, 0, sizeof(int) * (size_t)nt);
        for (long long jj = jstart[ii]; jj < jstart[ii + 1]; jj++) {      /* :580 */
            const int j = jflat[jj];
            const double delx = x[3 * j] - x[3 * i];                      /* :583-585 */
            const double dely = x[3 * j + 1] - x[3 * i + 1];
            const double delz = x[3 * j + 2] - x[3 * i + 2];
            const double rsq = delx * delx + dely * dely + delz * delz;   /* :586 */
            const int jtype = type_to_model[type[j] - 1] + 1;             /* :588 */
            if (rsq <= rc2) {                                             /* :589 */
                const int etnum = num_neigh[jtype - 1];
                num_neigh[jtype - 1] += 1;
                if (rsq < min_dR) min_dR = rsq;
                if (etnum >= m) {
                    overflow = 1;
                    continue;
                }
                const double rij = sqrt(rsq);
                const long long index = (long long)i * S + (long long)(jtype - 1) * m + etnum;
                dR[index * 4 + 0] = rij;
                dR[index * 4 + 1] = delx;
                dR[index * 4 + 2] = dely;
                dR[index * 4 + 3] = delz;
                list_neigh[index] = j + 1;
            }
        }
    }
    free(num_neigh);
    *min_rsq = min_dR;
    return overflow;
}
