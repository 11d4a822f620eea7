// qss_fortran_abi.h -- prototypes of the kernel-level entry points that keep
// the reference's Fortran calling convention (every argument by pointer,
// arrays column-major over the ghost box).  The GB300 library exports them so
// that the reference's own C drivers, and unit tests, can call single kernels.
#pragma once

#ifdef __cplusplus
extern "C" {
#endif

#define QSS_GB6 const int *, const int *, const int *, const int *, const int *, const int *

void getrhs3d2ndconst_(const double *phi, const double *vel_n, const double *b, double *max_H_over_dX,
                       double *lse_rhs, QSS_GB6, QSS_GB6, const double *dx, const double *dy,
                       const double *dz);
void getrhs3d3rdconst_(const double *phi, const double *vel_n, const double *b, double *max_H_over_dX,
                       double *lse_rhs, QSS_GB6, QSS_GB6, const double *dx, const double *dy,
                       const double *dz);
void getrhs3d2nd_(const double *phi, const double *vel_n, const double *b, const double *vel_x,
                  const double *vel_y, const double *vel_z, double *max_H_over_dX, double *lse_rhs,
                  QSS_GB6, QSS_GB6, const double *dx, const double *dy, const double *dz);
void getrhs3d3rd_(const double *phi, const double *vel_n, const double *b, const double *vel_x,
                  const double *vel_y, const double *vel_z, double *max_H_over_dX, double *lse_rhs,
                  QSS_GB6, QSS_GB6, const double *dx, const double *dy, const double *dz);
void getrhs3d5th_(const double *phi, const double *vel_n, const double *b, const double *vel_x,
                  const double *vel_y, const double *vel_z, double *max_H_over_dX, double *lse_rhs,
                  QSS_GB6, QSS_GB6, const double *dx, const double *dy, const double *dz);
void getcentralgrad3dorder2_(double *phi_x, double *phi_y, double *phi_z, QSS_GB6, const double *phi,
                             QSS_GB6, QSS_GB6, const double *dx, const double *dy, const double *dz);
void signedlinearextrapolation3d_(double *phi, QSS_GB6, QSS_GB6, const int *bdry_location_idx);
void setvarnorm3d_(const double *mask, const double *mask_x, const double *mask_y, const double *mask_z,
                   double *var_a, const double *a0, const double *ca, QSS_GB6, QSS_GB6,
                   const double *dx);
void setvarnorm3dtheta_(const double *mask, const double *mask_x, const double *mask_y,
                        const double *mask_z, double *var_a, const double *a0, const double *ca,
                        QSS_GB6, QSS_GB6, const double *dx);
void setvarcurvadv3d_(const double *mask, const double *mask_x, const double *mask_y,
                      const double *mask_z, double *var_b, double *vel_x, double *vel_y,
                      double *vel_z, double *b_max_over_dx, double *max_U_over_dx,
                      const double *const_b, QSS_GB6, QSS_GB6, const double *dx);
void qss3drk1step_(double *u_next, QSS_GB6, const double *u_cur, QSS_GB6, const double *rhs, QSS_GB6,
                   QSS_GB6, const double *dt);
void qss3dtvdrk2stage2_(double *u_stage2, QSS_GB6, const double *u_stage1, QSS_GB6,
                        const double *u_cur, QSS_GB6, const double *rhs, QSS_GB6, QSS_GB6,
                        const double *dt);
void qss3dtvdrk3stage3_(double *u_next, QSS_GB6, const double *u_stage2, QSS_GB6,
                        const double *u_cur, QSS_GB6, const double *rhs, QSS_GB6, QSS_GB6,
                        const double *dt);
void qss3dcomputedistanceforsubcellfix_(double *distance0, const double *phi0, QSS_GB6, QSS_GB6,
                                        const double *dx, const double *dy, const double *dz);
void qss3dcomputereinitializationeqnrhssubcellfixorder1_(double *reinit_rhs, const double *phi,
                                                         QSS_GB6, const double *phi0,
                                                         const double *distance0, QSS_GB6,
                                                         const double *dx, const double *dy,
                                                         const double *dz);
void qss3dmaxnormdifflocal_(double *max_norm_diff, const double *field1, QSS_GB6, const double *field2,
                            QSS_GB6, QSS_GB6, const double *local_zone);
void imposemaskparallel_(double *phi_masked, const double *mask, const double *phi,
                         const double *overlap, QSS_GB6, const int *cur_klo_gb, const int *cur_khi_gb);
void qss3dvolumeregionphilessthanzero_(double *volume, const double *phi, QSS_GB6, QSS_GB6,
                                       const double *dx, const double *dy, const double *dz,
                                       const double *epsilon);
void imposetrapvelocity3d_(const double *phi_w, const double *phi_nw, double *normal_velocity,
                           double *curvature_coeff, double *vel_x, double *vel_y, double *vel_z,
                           QSS_GB6, QSS_GB6, const double *dx);

#undef QSS_GB6

#ifdef __cplusplus
}
#endif
