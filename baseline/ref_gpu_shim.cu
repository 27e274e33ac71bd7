// Plain C entry points over two pieces of the reference's own GPU code, compiled unmodified from
// a staged copy of its sources: the LAMMPS NEP evaluator (class NEP3,
// src/lmps/lammps-libtorch/MATPL/NEP_GPU/force/nep3.cuh:90-180, nep3.cu:73-430 and :551-810)
// and the CalcOps_cuda force / virial launchers (src/op/include/calculate_force.h:1-30,
// src/op/kernel/calculateForce.cu:95-165, calculateVirial.cu:188-256).  They are the comparator
// the fused kernels are timed and checked against on the same GPU; nothing in the product links
// this library.
#include <cstdio>
#include <iostream>
#include <fcntl.h>
#include <unistd.h>

#include <cuda_runtime.h>

#include "nep3.cuh"
#include "calculate_force.h"

namespace {

// NEP3::init_from_file reports the model on stdout; keep it off the caller's stdout (a bench
// prints one JSON line there) by pointing fd 1 at /dev/null around the call.
struct QuietStdout {
  int saved = -1;
  QuietStdout() {
    fflush(stdout);
    std::cout.flush();
    int devnull = open("/dev/null", O_WRONLY);
    if (devnull >= 0) {
      saved = dup(1);
      dup2(devnull, 1);
      close(devnull);
    }
  }
  ~QuietStdout() {
    fflush(stdout);
    std::cout.flush();
    if (saved >= 0) {
      dup2(saved, 1);
      close(saved);
    }
  }
};

}  // namespace

extern "C" {

// Reads a nep.txt (nep5 format) and returns the evaluator, or NULL.  The reference exits the
// process on a malformed file.
void *refnep_create(const char *nep_txt, int device) {
  if (cudaSetDevice(device) != cudaSuccess) return nullptr;
  NEP3 *m = new NEP3();
  {
    QuietStdout q;
    m->init_from_file(nep_txt, false, device + 1);
  }
  return m;
}

void refnep_destroy(void *h) { delete static_cast<NEP3 *>(h); }

// Capacities of the per-atom radial / angular lists the evaluator filters into (the file's
// values x 1.25) and its cutoffs.  Its filter kernel writes as many entries as there are listed
// pairs inside each cutoff, without a bound check, and its sort kernel runs one thread per
// entry, so a caller checks those counts against these capacities (and the capacities against
// 1024) before the first call.
int refnep_capacity(void *h, int *mn_radial, int *mn_angular, float *rc_radial,
                    float *rc_angular) {
  NEP3 *m = static_cast<NEP3 *>(h);
  *mn_radial = m->paramb.MN_radial;
  *mn_angular = m->paramb.MN_angular;
  *rc_radial = m->paramb.rc_radial;
  *rc_angular = m->paramb.rc_angular;
  return 0;
}

// One PairMATPL::compute step of the GPU NEP path (pair_matpl.cpp:1093-1190): host arrays in,
// host energies / forces (SoA over local + ghost rows) / 6-component virial out; synchronous.
int refnep_compute(void *h, int build_neighbor, int n_all, int nlocal, int inum, int nm,
                   int *itype, int *ilist, int *numneigh, int *firstneigh, double *position,
                   double *ei, double *force, double *virial) {
  NEP3 *m = static_cast<NEP3 *>(h);
  m->compute_large_box_optim(build_neighbor != 0, n_all, nlocal, inum, nm, itype, ilist,
                             numneigh, firstneigh, position, ei, force, virial);
  return static_cast<int>(cudaGetLastError());
}

// CalcOps_cuda calculateForce / calculateVirial device launchers (the kernels the torch ops
// run after their own output set-up, CalcOps.cpp:6-22 and :170-186); dtype 0 = float64,
// 1 = float32.  The caller provides force already holding the centre term (zero ghost rows),
// and zeroed virial / atom_virial.
int refcalc_force(int dtype, const int *nblist, const void *dE, const void *Ri_d, int batch,
                  int natoms, int neigh_num, void *force, int nghost, int device) {
  if (dtype == 0)
    launch_calculate_force<double>(nblist, static_cast<const double *>(dE),
                                   static_cast<const double *>(Ri_d), batch, natoms, neigh_num,
                                   static_cast<double *>(force), nghost, device);
  else
    launch_calculate_force<float>(nblist, static_cast<const float *>(dE),
                                  static_cast<const float *>(Ri_d), batch, natoms, neigh_num,
                                  static_cast<float *>(force), nghost, device);
  return static_cast<int>(cudaGetLastError());
}

int refcalc_virial(int dtype, const int *nblist, const void *dE, const void *Rij,
                   const void *Ri_d, int batch, int natoms, int neigh_num, void *virial,
                   void *atom_virial, int nghost, int device) {
  if (dtype == 0)
    launch_calculate_virial_force<double>(
        nblist, static_cast<const double *>(dE), static_cast<const double *>(Rij),
        static_cast<const double *>(Ri_d), batch, natoms, neigh_num,
        static_cast<double *>(virial), static_cast<double *>(atom_virial), nghost, device);
  else
    launch_calculate_virial_force<float>(
        nblist, static_cast<const float *>(dE), static_cast<const float *>(Rij),
        static_cast<const float *>(Ri_d), batch, natoms, neigh_num, static_cast<float *>(virial),
        static_cast<float *>(atom_virial), nghost, device);
  return static_cast<int>(cudaGetLastError());
}

}  // extern "C"
