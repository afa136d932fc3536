/*
 * tvap_setup.h -- host-side model-space setup (no device code).
 *
 * These entry points restate the one-time initialisation that TAURUS_vap runs
 * before its gradient loop, so that a harness without the Fortran program can
 * build the inputs of the device path (include/tvap.h).  A Fortran caller of
 * the drop-in keeps its own set_basis/set_hamiltonian and never needs them.
 *
 *   tvs_load_antoine   set_basis (src/module_basis.f90:73-245) +
 *                      set_hamiltonian with hamil_read=0 for ANTOINE
 *                      JT files (src/module_hamiltonian.f90:79-401)
 *   tvs_synthetic      same pipeline fed by seeded N(0,1) JT elements
 *   tvs_write_red/     write_/read_hamiltonian_reduced
 *   tvs_read_red       (src/module_hamiltonian.f90:533-627)
 *   tvs_multipoles     set_multipoles (src/module_multipoles.f90:43-128)
 *   tvs_observable_ops set_angular_momentum (src/module_angularmomentum.f90:33-120),
 *                      set_radius (src/module_radius.f90:30-63) and the
 *                      single-particle parities of generate_rotation_parity
 *                      (src/module_projection.f90:607-625)
 *
 * All index arrays use the reference's values (1-based sp indices in abcd,
 * sp_sh and sp_tr).  Matrices are column-major; complex numbers are pairs of
 * doubles (re, im).
 */
#ifndef TVAP_SETUP_H
#define TVAP_SETUP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tvs_model tvs_model;

tvs_model* tvs_load_antoine(const char* path, double valence_Z, double valence_N);
tvs_model* tvs_synthetic(int nsh, const int* sh_na, const double* spe_p, const double* spe_n, double hw,
                         double core_Z, double core_N, double valence_Z, double valence_N,
                         unsigned long long seed, double scale, double damp);
const char* tvs_error(const tvs_model* m);
void tvs_free(tvs_model* m);

int tvs_dim(const tvs_model* m);
int tvs_nshells(const tvs_model* m);
long long tvs_nelements(const tvs_model* m);
double tvs_hw(const tvs_model* m);
double tvs_oscillator_length(const tvs_model* m);
void tvs_get_basis(const tvs_model* m, int* sp_n, int* sp_l, int* sp_2j, int* sp_2mj, int* sp_2mt, int* sp_sh,
                   int* sp_tr);
void tvs_get_shells(const tvs_model* m, int* sh_na);
void tvs_get_hamiltonian(const tvs_model* m, double* H0, double* H1, int16_t* abcd, float* h2, int8_t* trperm);
void tvs_multipoles(const tvs_model* m, double* q);
void tvs_coeff_betalm(const tvs_model* m, double* out);
/* ops: 9 * n * n doubles (Jx, Jy, Jz, Jx^2, Jy^2, Jz^2, spin-orbit, r^2 of
 * protons, r^2 of neutrons; vectorised as the reference's tables); parity: n. */
void tvs_observable_ops(const tvs_model* m, double* ops, int* parity);
int tvs_write_red(const tvs_model* m, const char* path);
int tvs_read_red(tvs_model* m, const char* path);
double tvs_clebsch(int j1, int j2, int j3, int m1, int m2, int m3);

#ifdef __cplusplus
}
#endif
#endif
