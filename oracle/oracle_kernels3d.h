/*
 * oracle_kernels3d.h -- TEST INFRASTRUCTURE (oracle).  Prototypes of the C
 * restatement of the reference's 3-D Fortran kernels (Fortran symbol names,
 * every argument by pointer).
 */
#ifndef ORACLE_KERNELS3D_H
#define ORACLE_KERNELS3D_H

#define O_GB const int *, const int *, const int *, const int *, const int *, const int *

void setvarnorm3d_(const double *, const double *, const double *, const double *, double *,
                   const double *, const double *, O_GB, O_GB, const double *);
void setvarnorm3dtheta_(const double *, const double *, const double *, const double *,
                        double *, const double *, const double *, O_GB, O_GB, const double *);
void setvarcurvadv3d_(const double *, const double *, const double *, const double *, double *,
                      double *, double *, double *, double *, double *, const double *, O_GB,
                      O_GB, const double *);
void getrhs3d2ndconst_(const double *, const double *, const double *, double *, double *,
                       O_GB, O_GB, const double *, const double *, const double *);
void getrhs3d3rdconst_(const double *, const double *, const double *, double *, double *,
                       O_GB, O_GB, const double *, const double *, const double *);
void getrhs3d2nd_(const double *, const double *, const double *, const double *,
                  const double *, const double *, double *, double *, O_GB, O_GB,
                  const double *, const double *, const double *);
void getrhs3d3rd_(const double *, const double *, const double *, const double *,
                  const double *, const double *, double *, double *, O_GB, O_GB,
                  const double *, const double *, const double *);
void getrhs3d5th_(const double *, const double *, const double *, const double *,
                  const double *, const double *, double *, double *, O_GB, O_GB,
                  const double *, const double *, const double *);
void getcentralgrad3dorder2_(double *, double *, double *, O_GB, const double *, O_GB, O_GB,
                             const double *, const double *, const double *);
void signedlinearextrapolation3d_(double *, O_GB, O_GB, const int *);
void qss3drk1step_(double *, O_GB, const double *, O_GB, const double *, O_GB, O_GB,
                   const double *);
void qss3dtvdrk2stage2_(double *, O_GB, const double *, O_GB, const double *, O_GB,
                        const double *, O_GB, O_GB, const double *);
void qss3dtvdrk3stage3_(double *, O_GB, const double *, O_GB, const double *, O_GB,
                        const double *, O_GB, O_GB, const double *);
void qss3dcomputedistanceforsubcellfix_(double *, const double *, O_GB, O_GB, const double *,
                                        const double *, const double *);
void qss3dcomputereinitializationeqnrhssubcellfixorder1_(double *, const double *, O_GB,
                                                         const double *, const double *, O_GB,
                                                         const double *, const double *,
                                                         const double *);
void qss3dmaxnormdifflocal_(double *, const double *, O_GB, const double *, O_GB, O_GB,
                            const double *);
void imposemaskparallel_(double *, const double *, const double *, const double *, O_GB,
                         const int *, const int *);
void imposemaskparallelvar_(double *, const double *, const double *, const double *, O_GB,
                            const int *, const int *);
void qss3dvolumeregionphilessthanzero_(double *, const double *, O_GB, O_GB, const double *,
                                       const double *, const double *, const double *);
void imposetrapvelocity3d_(const double *, const double *, double *, double *, double *,
                           double *, double *, O_GB, O_GB, const double *);

#undef O_GB
#endif
