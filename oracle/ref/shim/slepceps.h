/* Stand-in declarations for the SLEPc calls of ComputeLHSEigenvalues
 * (src/lhs.c:550-622).  TEST INFRASTRUCTURE ONLY; every call fails, the
 * function is never invoked by the harness. */
#ifndef CH_SLEPC_STANDIN_H
#define CH_SLEPC_STANDIN_H
#include "petsc.h"

typedef struct _p_EPS* EPS;
typedef const char* EPSType;
typedef enum { EPS_HEP = 1 } EPSProblemType;
typedef enum { EPS_ERROR_ABSOLUTE, EPS_ERROR_RELATIVE } EPSErrorType;

PetscErrorCode EPSCreate(MPI_Comm c, EPS* e);
PetscErrorCode EPSSetOperators(EPS e, Mat A, Mat B);
PetscErrorCode EPSSetProblemType(EPS e, EPSProblemType t);
PetscErrorCode EPSSetFromOptions(EPS e);
PetscErrorCode EPSSolve(EPS e);
PetscErrorCode EPSGetIterationNumber(EPS e, PetscInt* its);
PetscErrorCode EPSGetType(EPS e, EPSType* t);
PetscErrorCode EPSGetDimensions(EPS e, PetscInt* nev, PetscInt* ncv, PetscInt* mpd);
PetscErrorCode EPSGetTolerances(EPS e, PetscReal* tol, PetscInt* maxit);
PetscErrorCode EPSGetConverged(EPS e, PetscInt* nconv);
PetscErrorCode EPSGetEigenpair(EPS e, PetscInt i, PetscScalar* kr, PetscScalar* ki, Vec xr, Vec xi);
PetscErrorCode EPSComputeError(EPS e, PetscInt i, EPSErrorType t, PetscReal* err);
PetscErrorCode EPSDestroy(EPS* e);
#endif
