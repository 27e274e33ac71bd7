/*
 * ORACLE — test infrastructure only.  Never linked into, loaded by or called from
 * the product library; only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg use it, to check results and to time the CPU baseline.
 *
 * Plain-C restatement of MatPL's DP neighbor search
 *   src/pre_data/gen_feature/NeighConst.f90:14-149  (subroutine find_neighbore)
 * and of the radial column of the ImageDR tensor built by
 *   src/pre_data/dpuni_data_loader.py:595-650 (find_neighbore) and :652-716 (compute_Ri).
 *
 * The Fortran module cannot be built here (it needs ifort + MKL), so this file is the
 * executable statement of its semantics.  Floating-point evaluation order follows the
 * Fortran source left to right with no fused multiply-add; this file must be compiled
 * with -ffp-contract=off so that gcc on x86_64 and aarch64 gives the same bits.
 *
 * Layouts (row-major, C order, already transposed the way the Python loader does it):
 *   lattice    [images][3][3]  lattice[n][v][k] = component k of lattice vector v
 *   position   [images][natoms][3] fractional; wrapped in place by mod(x+10,1) as Fortran does
 *   type_maps  [natoms]         1-based type index of each atom
 *   Rc_type    [ntypes]         per centre-type cutoff
 *   list_neigh [images][natoms][ntypes][m_neigh]  1-based neighbor index, 0 = empty
 *   dR_neigh   [images][natoms][ntypes][m_neigh][3]
 * Return: 0 on success, 1 when a type block would exceed m_neigh (the Fortran "stop").
 */
#include <math.h>
#include <string.h>
#include <stdint.h>

static double fortran_mod1(double a) { return fmod(a, 1.0); }

static void mic_component(double *d) {
    /* NeighConst.f90:99-100 — two sequential nearest-image corrections */
    if (fabs(*d + 1.0) < fabs(*d)) *d = *d + 1.0;
    if (fabs(*d - 1.0) < fabs(*d)) *d = *d - 1.0;
}

int matpl_oracle_find_neighbore(int images, const double *lattice, double *position,
                                int ntypes, int natoms, int m_neigh, double Rc_M,
                                const double *Rc_type, const int *type_maps,
                                int32_t *list_neigh, double *dR_neigh)
{
    const long long slots_per_atom = (long long)ntypes * m_neigh;
    memset(list_neigh, 0, sizeof(int32_t) * (size_t)images * natoms * slots_per_atom);
    memset(dR_neigh, 0, sizeof(double) * 3 * (size_t)images * natoms * slots_per_atom);
    int iflag = 0; /* NeighConst.f90:35 — set once, never reset between images */
    int overflow = 0;
    if (ntypes > 64) return 2;

    for (int n = 0; n < images; ++n) {
        const double *L = lattice + 9 * n;
        double *P = position + (size_t)3 * natoms * n;
        int nperiod[3];
        for (int v = 0; v < 3; ++v) {
            double d = sqrt(L[3 * v + 0] * L[3 * v + 0] + L[3 * v + 1] * L[3 * v + 1]
                            + L[3 * v + 2] * L[3 * v + 2]);
            nperiod[v] = (int)(Rc_M / d) + 1;
            if (d < 2 * Rc_M) iflag = 1;
        }
        for (int i = 0; i < natoms; ++i)
            for (int k = 0; k < 3; ++k) P[3 * i + k] = fortran_mod1(P[3 * i + k] + 10.0);

        const double Rc2 = Rc_M * Rc_M;
        /* centre atoms are independent: with OpenMP they run in parallel (each writes only its
         * own rows); the Fortran "stop" becomes a flag that ends that atom's search */
#pragma omp parallel for schedule(dynamic, 16) reduction(|| : overflow)
        for (int i = 0; i < natoms; ++i) {
            int num_type[64], num_type_M[64];
            const double rct = Rc_type[type_maps[i] - 1];
            const double rct2 = rct * rct;
            int32_t *LN = list_neigh + ((size_t)n * natoms + i) * slots_per_atom;
            double *DR = dR_neigh + 3 * ((size_t)n * natoms + i) * slots_per_atom;
            int stop = 0;
            for (int t = 0; t < ntypes; ++t) { num_type[t] = 0; num_type_M[t] = 0; }
            for (int j = 0; j < natoms && !stop; ++j) {
                int ilo[3], ihi[3];
                for (int v = 0; v < 3; ++v) {
                    ilo[v] = iflag ? -nperiod[v] : 0;
                    ihi[v] = iflag ? nperiod[v] : 0;
                }
                for (int i1 = ilo[0]; i1 <= ihi[0] && !stop; ++i1)
                for (int i2 = ilo[1]; i2 <= ihi[1] && !stop; ++i2)
                for (int i3 = ilo[2]; i3 <= ihi[2] && !stop; ++i3) {
                    double dx1, dx2, dx3;
                    if (iflag) { /* NeighConst.f90:62-64 */
                        dx1 = P[3 * j + 0] - P[3 * i + 0] + i1;
                        dx2 = P[3 * j + 1] - P[3 * i + 1] + i2;
                        dx3 = P[3 * j + 2] - P[3 * i + 2] + i3;
                    } else {     /* NeighConst.f90:98-108 */
                        dx1 = P[3 * j + 0] - P[3 * i + 0]; mic_component(&dx1);
                        dx2 = P[3 * j + 1] - P[3 * i + 1]; mic_component(&dx2);
                        dx3 = P[3 * j + 2] - P[3 * i + 2]; mic_component(&dx3);
                    }
                    const double dx = L[0] * dx1 + L[3] * dx2 + L[6] * dx3;
                    const double dy = L[1] * dx1 + L[4] * dx2 + L[7] * dx3;
                    const double dz = L[2] * dx1 + L[5] * dx2 + L[8] * dx3;
                    const double dd = dx * dx + dy * dy + dz * dz;
                    if (dd < Rc2 && dd > 1.0e-8) {
                        const int it = type_maps[j] - 1;
                        num_type_M[it] += 1;
                        if (num_type_M[it] > m_neigh) { stop = 1; overflow = 1; break; }
                        if (dd < rct2 && dd > 1.0e-8) {
                            const int slot = it * m_neigh + num_type[it];
                            num_type[it] += 1;
                            LN[slot] = j + 1;
                            DR[3 * slot + 0] = dx;
                            DR[3 * slot + 1] = dy;
                            DR[3 * slot + 2] = dz;
                        }
                    }
                }
            }
        }
        if (overflow) return 1;
        /* NeighConst.f90:136-147 — clear slots whose |dR|_1 <= 1e-8 */
#pragma omp parallel for schedule(static)
        for (int i = 0; i < natoms; ++i) {
            int32_t *LN = list_neigh + ((size_t)n * natoms + i) * slots_per_atom;
            double *DR = dR_neigh + 3 * ((size_t)n * natoms + i) * slots_per_atom;
            for (long long s = 0; s < slots_per_atom; ++s) {
                if (fabs(DR[3 * s]) + fabs(DR[3 * s + 1]) + fabs(DR[3 * s + 2]) <= 1.0e-8) {
                    LN[s] = 0; DR[3 * s] = 0; DR[3 * s + 1] = 0; DR[3 * s + 2] = 0;
                }
            }
        }
    }
    return 0;
}

/* dpuni_data_loader.py:669-673 — r = sqrt(dx*dx + dy*dy + dz*dz) where list_neigh > 0,
 * then ImageDR = concat(r, dR) along the last axis. */
void matpl_oracle_image_dr(long long nslots, const int32_t *list_neigh, const double *dR,
                           double *image_dr)
{
    for (long long s = 0; s < nslots; ++s) {
        double r = 0.0;
        if (list_neigh[s] > 0) {
            const double x = dR[3 * s], y = dR[3 * s + 1], z = dR[3 * s + 2];
            r = sqrt(x * x + y * y + z * z);
        }
        image_dr[4 * s + 0] = r;
        image_dr[4 * s + 1] = dR[3 * s + 0];
        image_dr[4 * s + 2] = dR[3 * s + 1];
        image_dr[4 * s + 3] = dR[3 * s + 2];
    }
}
