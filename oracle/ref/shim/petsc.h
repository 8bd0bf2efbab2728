/*
 * Minimal stand-in for the subset of PETSc that the reference's hot-path
 * sources call (src/particles.c, src/lhs.c, src/rhs.c, src/calculus.c,
 * src/vectors.c, src/random.c).  TEST INFRASTRUCTURE ONLY: it lets those
 * sources compile unmodified, single process, so that their outputs pin
 * the oracle.  Semantics implemented: periodic DMDA with ghost width 1 and
 * box stencil, global/local vectors, DMDAVecGetArray index tables,
 * GlobalToLocal (INSERT), LocalToGlobal (ADD folds ghosts periodically),
 * VecStrideGather, field decomposition, MatSetValuesStencil row capture,
 * constant null-space removal, and a DMSwarm holding user struct fields.
 */
#ifndef CH_PETSC_STANDIN_H
#define CH_PETSC_STANDIN_H

#include <float.h>
#include <stddef.h>
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

typedef double PetscReal;
typedef double PetscScalar;
typedef int PetscInt;
typedef int PetscMPIInt;
typedef int PetscErrorCode;
typedef int PetscEnum;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef long PetscLogDouble;
typedef int MPI_Comm;

#define PETSC_SUCCESS 0
#define PETSC_COMM_WORLD 0
#define PETSC_STDOUT stdout
#define PETSC_VIEWER_STDOUT_WORLD ((PetscViewer)0)
#define PETSC_MAX_PATH_LEN 4096
#define PETSC_DECIDE (-1)
#define PETSC_PI 3.14159265358979323846
#define PETSC_MACHINE_EPSILON DBL_EPSILON

#define PETSC_ERR_ARG_WRONG 62
#define PETSC_ERR_ARG_UNKNOWN_TYPE 86
#define PETSC_ERR_ARG_INCOMP 75
#define PETSC_ERR_SIG 59
#define PETSC_ERR_SUP 56
#define PETSC_ERR_LIB 76
#define PETSC_ERR_ARG_OUTOFRANGE 63
#define PETSC_ERR_ORDER 73

typedef enum { INSERT_VALUES = 1, ADD_VALUES = 2 } InsertMode;
typedef enum { MAT_FLUSH_ASSEMBLY = 1, MAT_FINAL_ASSEMBLY = 0 } MatAssemblyType;
typedef enum { DM_BOUNDARY_NONE, DM_BOUNDARY_GHOSTED, DM_BOUNDARY_MIRROR, DM_BOUNDARY_PERIODIC,
               DM_BOUNDARY_TWIST } DMBoundaryType;
typedef enum { DMDA_STENCIL_STAR, DMDA_STENCIL_BOX } DMDAStencilType;
typedef enum { FILE_MODE_READ, FILE_MODE_WRITE } PetscFileMode;

typedef struct { PetscInt k, j, i, c; } MatStencil;

typedef struct _p_DM* DM;
typedef struct _p_Vec* Vec;
typedef struct _p_Mat* Mat;
typedef struct _p_KSP* KSP;
typedef struct _p_MatNullSpace* MatNullSpace;
typedef struct _p_PetscViewer* PetscViewer;
typedef struct _p_PetscObject* PetscObject;
typedef struct _p_PetscOptions* PetscOptions;
typedef const char* KSPType;
#define KSPCG "cg"
#define KSPBCGS "bcgs"
#define KSPGMRES "gmres"

extern int ch_standin_verbose;
int ch_standin_error(int code, const char* func, const char* fmt, ...);

#define PetscFunctionBeginUser do { } while (0)
#define PetscFunctionReturn(x) return (x)
#define PetscCall(x) do { PetscErrorCode ierr__ = (x); if (ierr__) return ierr__; } while (0)
#define PetscCallMPI(x) PetscCall(x)
#define SETERRQ(comm, code, ...) return ch_standin_error((code), __func__, __VA_ARGS__)
#define PetscFree(p) (free(p), (p) = NULL, 0)

#define PetscSqr(x) ((x) * (x))
#define PetscSqrtReal(x) sqrt(x)
#define PetscCosReal(x) cos(x)
#define PetscSinReal(x) sin(x)
#define PetscCosScalar(x) cos(x)
#define PetscSinScalar(x) sin(x)
#define PetscAbsReal(x) fabs(x)
#define PetscLog10Real(x) log10(x)
#define PetscMax(a, b) ((a) > (b) ? (a) : (b))
#define PetscMin(a, b) ((a) < (b) ? (a) : (b))
#define PetscRealPart(x) (x)
#define PetscImaginaryPart(x) (0.0)

int MPI_Comm_size(MPI_Comm comm, PetscMPIInt* size);
PetscErrorCode PetscPrintf(MPI_Comm comm, const char* fmt, ...);
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm comm, const char* fmt, ...);
PetscErrorCode PetscSynchronizedFlush(MPI_Comm comm, FILE* f);
PetscErrorCode PetscStrcmp(const char* a, const char* b, PetscBool* flg);
PetscErrorCode PetscStrcat(char* a, const char* b);
PetscErrorCode PetscObjectSetName(PetscObject obj, const char* name);
PetscErrorCode PetscObjectSetOptionsPrefix(PetscObject obj, const char* prefix);

/* Vec */
PetscErrorCode VecZeroEntries(Vec v);
PetscErrorCode VecSet(Vec v, PetscScalar a);
PetscErrorCode VecMean(Vec v, PetscScalar* m);
PetscErrorCode VecDestroy(Vec* v);
PetscErrorCode VecStrideGather(Vec full, PetscInt field, Vec s, InsertMode mode);
PetscErrorCode VecGetArray(Vec v, PetscScalar** a);
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a);

/* DM / DMDA */
PetscErrorCode DMGetLocalVector(DM dm, Vec* v);
PetscErrorCode DMRestoreLocalVector(DM dm, Vec* v);
PetscErrorCode DMGetGlobalVector(DM dm, Vec* v);
PetscErrorCode DMRestoreGlobalVector(DM dm, Vec* v);
PetscErrorCode DMCreateGlobalVector(DM dm, Vec* v);
PetscErrorCode DMGlobalToLocal(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMGlobalToLocalBegin(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMGlobalToLocalEnd(DM dm, Vec g, InsertMode mode, Vec l);
PetscErrorCode DMLocalToGlobal(DM dm, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMLocalToGlobalBegin(DM dm, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMLocalToGlobalEnd(DM dm, Vec l, InsertMode mode, Vec g);
PetscErrorCode DMDAVecGetArray(DM dm, Vec v, void* array);
PetscErrorCode DMDAVecRestoreArray(DM dm, Vec v, void* array);
PetscErrorCode DMDAGetCorners(DM dm, PetscInt* x, PetscInt* y, PetscInt* z, PetscInt* m, PetscInt* n, PetscInt* p);
PetscErrorCode DMCreateFieldDecomposition(DM dm, PetscInt* nf, char*** names, void* is, DM** dms);
PetscErrorCode DMDestroy(DM* dm);
PetscErrorCode DMView(DM dm, PetscViewer v);
PetscErrorCode DMGetDimension(DM dm, PetscInt* dim);

/* DMSwarm */
#define DMSwarmPICField_coor "DMSwarmPIC_coor"
PetscErrorCode DMSwarmGetCellDM(DM sw, DM* dm);
PetscErrorCode DMSwarmGetField(DM sw, const char* name, PetscInt* bs, void* type, void** data);
PetscErrorCode DMSwarmRestoreField(DM sw, const char* name, PetscInt* bs, void* type, void** data);
PetscErrorCode DMSwarmGetLocalSize(DM sw, PetscInt* n);
PetscErrorCode DMSwarmGetSize(DM sw, PetscInt* n);
PetscErrorCode DMSwarmMigrate(DM sw, PetscBool remove);

/* Mat / KSP */
PetscErrorCode MatSetValuesStencil(Mat A, PetscInt m, const MatStencil* rows, PetscInt n, const MatStencil* cols,
                                   const PetscScalar* v, InsertMode mode);
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t);
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t);
PetscErrorCode MatZeroEntries(Mat A);
PetscErrorCode MatShift(Mat A, PetscScalar a);
PetscErrorCode MatView(Mat A, PetscViewer v);
PetscErrorCode MatCreateVecs(Mat A, Vec* r, Vec* l);
PetscErrorCode MatNullSpaceCreate(MPI_Comm c, PetscBool has_cnst, PetscInt n, const Vec* vecs, MatNullSpace* sp);
PetscErrorCode MatSetNullSpace(Mat A, MatNullSpace sp);
PetscErrorCode MatNullSpaceDestroy(MatNullSpace* sp);
PetscErrorCode MatNullSpaceRemove(MatNullSpace sp, Vec v);
PetscErrorCode KSPGetDM(KSP ksp, DM* dm);
PetscErrorCode KSPGetSolution(KSP ksp, Vec* v);
PetscErrorCode KSPGetOperators(KSP ksp, Mat* A, Mat* P);
PetscErrorCode KSPGetTolerances(KSP ksp, PetscReal* rtol, PetscReal* abstol, PetscReal* dtol, PetscInt* maxits);
PetscErrorCode KSPGetType(KSP ksp, KSPType* type);
/* Options database (PetscOptionsGet*; NULL database = the global one) */
PetscErrorCode PetscOptionsGetString(PetscOptions o, const char pre[], const char name[], char str[], size_t len,
                                     PetscBool* set);
PetscErrorCode PetscOptionsGetInt(PetscOptions o, const char pre[], const char name[], PetscInt* v, PetscBool* set);
PetscErrorCode PetscOptionsGetReal(PetscOptions o, const char pre[], const char name[], PetscReal* v,
                                   PetscBool* set);
PetscErrorCode PetscOptionsHasName(PetscOptions o, const char pre[], const char name[], PetscBool* set);
PetscErrorCode PetscViewerBinaryOpen(MPI_Comm c, const char* name, PetscFileMode m, PetscViewer* v);
PetscErrorCode PetscViewerDestroy(PetscViewer* v);

#endif
