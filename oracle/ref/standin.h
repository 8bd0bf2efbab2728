/* Constructors of the PETSc stand-in objects used by the reference harness.
 * TEST INFRASTRUCTURE ONLY. */
#ifndef CH_STANDIN_PRIV_H
#define CH_STANDIN_PRIV_H
#include "shim/petsc.h"

struct _p_DM {
  int is_swarm;
  int Nx, Ny, Nz, dof, sw;
  char* fieldnames[8];
  DM celldm;              /* swarm: the cell DM */
  int np;                 /* swarm: local size */
  void* position;         /* swarm: RealVector[np] */
  void* velocity;         /* swarm: RealVector[np] */
  double* coor;           /* swarm: DMSwarmPIC_coor [np*3] */
};

struct _p_Vec {
  DM dm;
  int local;              /* ghosted local vector */
  int n;                  /* scalars */
  double* a;
  void** tables;          /* index tables handed out by DMDAVecGetArray */
  void* array_ptr;
  char name[64];
};

struct _p_Mat {
  int N;                  /* rows */
  int* ncols;             /* N */
  int* cols;              /* N x 27 */
  double* vals;           /* N x 27 */
};

struct _p_KSP {
  DM dm;
  Vec sol;
  Mat A;
  char type[32];          /* KSPSetType / -ksp_type (PETSc's default: gmres) */
  double rtol, abstol, dtol;
  int maxits;
};

DM ch_standin_dmda(int Nx, int Ny, int Nz, int dof, const char* const* names);
DM ch_standin_swarm(DM celldm, int np);
Mat ch_standin_mat(int N);
void ch_standin_mat_free(Mat A);
Vec ch_standin_global(DM dm);
/* A KSP whose type and tolerances are those KSPSetFromOptions would set
 * from the options database (-ksp_type, -ksp_rtol, -ksp_atol, -ksp_max_it),
 * on PETSc's defaults (gmres, 1e-5, 1e-50, 1e4, 10000). */
KSP ch_standin_ksp(DM dm);
/* Replaces the options database with argv[0..argc) ("-name value" pairs,
 * or a lone "-name"). */
void ch_standin_options(int argc, const char* const* argv);
#endif
