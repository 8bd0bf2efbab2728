/*
 * standin.c -- the PETSc/SLEPc stand-in behind oracle/ref/shim.
 * TEST INFRASTRUCTURE ONLY (see shim/petsc.h).  Single process, periodic
 * DMDA, ghost width 1, box stencil.
 */
#include "standin.h"

#include <stdarg.h>

#include "shim/slepceps.h"

int ch_standin_verbose = 0;

int ch_standin_error(int code, const char* func, const char* fmt, ...) {
  if (ch_standin_verbose) {
    va_list ap;
    va_start(ap, fmt);
    fprintf(stderr, "[standin] %s: ", func);
    vfprintf(stderr, fmt, ap);
    fprintf(stderr, "\n");
    va_end(ap);
  }
  return code;
}

PetscErrorCode PetscPrintf(MPI_Comm c, const char* fmt, ...) {
  (void)c;
  if (ch_standin_verbose) {
    va_list ap;
    va_start(ap, fmt);
    vfprintf(stderr, fmt, ap);
    va_end(ap);
  }
  return 0;
}
int MPI_Comm_size(MPI_Comm comm, PetscMPIInt* size) { (void)comm; *size = 1; return 0; }
PetscErrorCode PetscSynchronizedPrintf(MPI_Comm c, const char* fmt, ...) { (void)c; (void)fmt; return 0; }
PetscErrorCode PetscSynchronizedFlush(MPI_Comm c, FILE* f) { (void)c; (void)f; return 0; }
PetscErrorCode PetscStrcmp(const char* a, const char* b, PetscBool* flg) {
  *flg = (a && b && strcmp(a, b) == 0) ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}
PetscErrorCode PetscStrcat(char* a, const char* b) { strcat(a, b); return 0; }
PetscErrorCode PetscObjectSetName(PetscObject o, const char* name) { (void)o; (void)name; return 0; }
PetscErrorCode PetscObjectSetOptionsPrefix(PetscObject o, const char* p) { (void)o; (void)p; return 0; }

/* ---------------- objects ---------------- */
DM ch_standin_dmda(int Nx, int Ny, int Nz, int dof, const char* const* names) {
  DM dm = (DM)calloc(1, sizeof(*dm));
  dm->Nx = Nx; dm->Ny = Ny; dm->Nz = Nz; dm->dof = dof; dm->sw = 1;
  for (int f = 0; f < dof && f < 8; ++f) {
    const char* nm = names ? names[f] : "field";
    dm->fieldnames[f] = strdup(nm);
  }
  return dm;
}

DM ch_standin_swarm(DM celldm, int np) {
  DM sw = (DM)calloc(1, sizeof(*sw));
  sw->is_swarm = 1;
  sw->celldm = celldm;
  sw->np = np;
  sw->position = calloc((size_t)np, 4 * sizeof(double));
  sw->velocity = calloc((size_t)np, 4 * sizeof(double));
  sw->coor = (double*)calloc((size_t)np, 3 * sizeof(double));
  return sw;
}

Mat ch_standin_mat(int N) {
  Mat A = (Mat)calloc(1, sizeof(*A));
  A->N = N;
  A->ncols = (int*)calloc((size_t)N, sizeof(int));
  A->cols = (int*)calloc((size_t)N * 27, sizeof(int));
  A->vals = (double*)calloc((size_t)N * 27, sizeof(double));
  return A;
}

void ch_standin_mat_free(Mat A) {
  if (!A) return;
  free(A->ncols); free(A->cols); free(A->vals); free(A);
}

static Vec newvec(DM dm, int local) {
  Vec v = (Vec)calloc(1, sizeof(*v));
  v->dm = dm;
  v->local = local;
  int s = local ? 2 * dm->sw : 0;
  v->n = (dm->Nx + s) * (dm->Ny + s) * (dm->Nz + s) * dm->dof;
  v->a = (double*)calloc((size_t)v->n, sizeof(double));
  return v;
}

Vec ch_standin_global(DM dm) { return newvec(dm, 0); }

static void freevec(Vec v) {
  if (!v) return;
  free(v->tables);
  free(v->a);
  free(v);
}

PetscErrorCode VecZeroEntries(Vec v) { memset(v->a, 0, sizeof(double) * v->n); return 0; }
PetscErrorCode VecSet(Vec v, PetscScalar a) { for (int i = 0; i < v->n; ++i) v->a[i] = a; return 0; }
PetscErrorCode VecMean(Vec v, PetscScalar* m) {
  double s = 0.0;
  for (int i = 0; i < v->n; ++i) s += v->a[i];
  *m = s / v->n;
  return 0;
}
PetscErrorCode VecDestroy(Vec* v) { if (v && *v) { freevec(*v); *v = NULL; } return 0; }
PetscErrorCode VecGetArray(Vec v, PetscScalar** a) { *a = v->a; return 0; }
PetscErrorCode VecRestoreArray(Vec v, PetscScalar** a) { (void)v; *a = NULL; return 0; }

PetscErrorCode VecStrideGather(Vec full, PetscInt field, Vec s, InsertMode mode) {
  int dof = full->dm->dof, n = full->n / dof;
  for (int i = 0; i < n; ++i) {
    if (mode == ADD_VALUES) s->a[i] += full->a[i * dof + field];
    else s->a[i] = full->a[i * dof + field];
  }
  return 0;
}

PetscErrorCode DMGetLocalVector(DM dm, Vec* v) { *v = newvec(dm, 1); return 0; }
PetscErrorCode DMRestoreLocalVector(DM dm, Vec* v) { (void)dm; freevec(*v); *v = NULL; return 0; }
PetscErrorCode DMGetGlobalVector(DM dm, Vec* v) { *v = newvec(dm, 0); return 0; }
PetscErrorCode DMRestoreGlobalVector(DM dm, Vec* v) { (void)dm; freevec(*v); *v = NULL; return 0; }
PetscErrorCode DMCreateGlobalVector(DM dm, Vec* v) { *v = newvec(dm, 0); return 0; }

static inline int wrapi(int i, int n) { i %= n; return i < 0 ? i + n : i; }

/* local (ghosted) offset of node (i, j, k), i in [-sw, N+sw) */
static inline int loff(DM dm, int i, int j, int k) {
  int s = dm->sw, gx = dm->Nx + 2 * s, gy = dm->Ny + 2 * s;
  return (((k + s) * gy + (j + s)) * gx + (i + s)) * dm->dof;
}
static inline int goff(DM dm, int i, int j, int k) {
  return ((wrapi(k, dm->Nz) * dm->Ny + wrapi(j, dm->Ny)) * dm->Nx + wrapi(i, dm->Nx)) * dm->dof;
}

PetscErrorCode DMGlobalToLocal(DM dm, Vec g, InsertMode mode, Vec l) {
  int s = dm->sw;
  for (int k = -s; k < dm->Nz + s; ++k)
    for (int j = -s; j < dm->Ny + s; ++j)
      for (int i = -s; i < dm->Nx + s; ++i)
        for (int c = 0; c < dm->dof; ++c) {
          double v = g->a[goff(dm, i, j, k) + c];
          if (mode == ADD_VALUES) l->a[loff(dm, i, j, k) + c] += v;
          else l->a[loff(dm, i, j, k) + c] = v;
        }
  return 0;
}
PetscErrorCode DMGlobalToLocalBegin(DM dm, Vec g, InsertMode m, Vec l) { return DMGlobalToLocal(dm, g, m, l); }
PetscErrorCode DMGlobalToLocalEnd(DM dm, Vec g, InsertMode m, Vec l) { (void)dm; (void)g; (void)m; (void)l; return 0; }

/* ADD_VALUES adds every local entry, ghosts included, to its periodic
 * owner; INSERT_VALUES copies the owned part only. */
PetscErrorCode DMLocalToGlobal(DM dm, Vec l, InsertMode mode, Vec g) {
  int s = dm->sw;
  if (mode == INSERT_VALUES) {
    for (int k = 0; k < dm->Nz; ++k)
      for (int j = 0; j < dm->Ny; ++j)
        for (int i = 0; i < dm->Nx; ++i)
          for (int c = 0; c < dm->dof; ++c) g->a[goff(dm, i, j, k) + c] = l->a[loff(dm, i, j, k) + c];
    return 0;
  }
  for (int k = -s; k < dm->Nz + s; ++k)
    for (int j = -s; j < dm->Ny + s; ++j)
      for (int i = -s; i < dm->Nx + s; ++i)
        for (int c = 0; c < dm->dof; ++c) g->a[goff(dm, i, j, k) + c] += l->a[loff(dm, i, j, k) + c];
  return 0;
}
PetscErrorCode DMLocalToGlobalBegin(DM dm, Vec l, InsertMode m, Vec g) { return DMLocalToGlobal(dm, l, m, g); }
PetscErrorCode DMLocalToGlobalEnd(DM dm, Vec l, InsertMode m, Vec g) { (void)dm; (void)l; (void)m; (void)g; return 0; }

/* Index tables such that a[k][j][i] addresses node (i, j, k) in units of
 * dof scalars, like DMDAVecGetArray on a (possibly ghosted) vector. */
PetscErrorCode DMDAVecGetArray(DM dm, Vec v, void* array) {
  int s = v->local ? dm->sw : 0;
  int gx = dm->Nx + 2 * s, gy = dm->Ny + 2 * s, gz = dm->Nz + 2 * s;
  free(v->tables);
  v->tables = (void**)calloc((size_t)gz + (size_t)gz * gy, sizeof(void*));
  double*** planes = (double***)v->tables;
  double** rows = (double**)(v->tables + gz);
  for (int kk = 0; kk < gz; ++kk) {
    for (int jj = 0; jj < gy; ++jj)
      rows[kk * gy + jj] = v->a + ((size_t)(kk * gy + jj) * gx) * dm->dof + (ptrdiff_t)s * dm->dof;
    planes[kk] = &rows[kk * gy] + s;
  }
  *(double****)array = planes + s;
  return 0;
}
PetscErrorCode DMDAVecRestoreArray(DM dm, Vec v, void* array) {
  (void)dm;
  free(v->tables);
  v->tables = NULL;
  *(void**)array = NULL;
  return 0;
}
PetscErrorCode DMDAGetCorners(DM dm, PetscInt* x, PetscInt* y, PetscInt* z, PetscInt* m, PetscInt* n, PetscInt* p) {
  *x = 0; *y = 0; *z = 0; *m = dm->Nx; *n = dm->Ny; *p = dm->Nz;
  return 0;
}
PetscErrorCode DMCreateFieldDecomposition(DM dm, PetscInt* nf, char*** names, void* is, DM** dms) {
  (void)is;
  *nf = dm->dof;
  *names = (char**)calloc((size_t)dm->dof, sizeof(char*));
  *dms = (DM*)calloc((size_t)dm->dof, sizeof(DM));
  for (int f = 0; f < dm->dof; ++f) {
    (*names)[f] = strdup(dm->fieldnames[f] ? dm->fieldnames[f] : "");
    (*dms)[f] = ch_standin_dmda(dm->Nx, dm->Ny, dm->Nz, 1, NULL);
  }
  return 0;
}
PetscErrorCode DMDestroy(DM* dm) {
  if (dm && *dm) {
    for (int f = 0; f < 8; ++f) free((*dm)->fieldnames[f]);
    if ((*dm)->is_swarm) { free((*dm)->position); free((*dm)->velocity); free((*dm)->coor); }
    free(*dm);
    *dm = NULL;
  }
  return 0;
}
PetscErrorCode DMView(DM dm, PetscViewer v) { (void)dm; (void)v; return 0; }
PetscErrorCode DMGetDimension(DM dm, PetscInt* dim) { (void)dm; *dim = 3; return 0; }

/* ---------------- swarm ---------------- */
PetscErrorCode DMSwarmGetCellDM(DM sw, DM* dm) { *dm = sw->celldm; return 0; }
PetscErrorCode DMSwarmGetField(DM sw, const char* name, PetscInt* bs, void* type, void** data) {
  (void)bs; (void)type;
  if (!strcmp(name, "position")) *data = sw->position;
  else if (!strcmp(name, "velocity")) *data = sw->velocity;
  else if (!strcmp(name, DMSwarmPICField_coor)) *data = sw->coor;
  else return ch_standin_error(PETSC_ERR_ARG_WRONG, __func__, "no field %s", name);
  return 0;
}
PetscErrorCode DMSwarmRestoreField(DM sw, const char* name, PetscInt* bs, void* type, void** data) {
  (void)sw; (void)name; (void)bs; (void)type;
  *data = NULL;
  return 0;
}
PetscErrorCode DMSwarmGetLocalSize(DM sw, PetscInt* n) { *n = sw->np; return 0; }
PetscErrorCode DMSwarmGetSize(DM sw, PetscInt* n) { *n = sw->np; return 0; }
PetscErrorCode DMSwarmMigrate(DM sw, PetscBool remove) { (void)sw; (void)remove; return 0; }

/* ---------------- Mat / KSP ---------------- */
PetscErrorCode MatSetValuesStencil(Mat A, PetscInt m, const MatStencil* rows, PetscInt n, const MatStencil* cols,
                                   const PetscScalar* v, InsertMode mode) {
  /* the stand-in only records rows of the potential DMDA (dof 1) */
  extern DM ch_standin_matdm;
  DM dm = ch_standin_matdm;
  for (int r = 0; r < m; ++r) {
    int row = goff(dm, rows[r].i, rows[r].j, rows[r].k);
    for (int c = 0; c < n; ++c) {
      int col = goff(dm, cols[c].i, cols[c].j, cols[c].k);
      int q, found = -1;
      for (q = 0; q < A->ncols[row]; ++q)
        if (A->cols[row * 27 + q] == col) { found = q; break; }
      if (found < 0) {
        found = A->ncols[row]++;
        A->cols[row * 27 + found] = col;
        A->vals[row * 27 + found] = 0.0;
      }
      if (mode == ADD_VALUES) A->vals[row * 27 + found] += v[r * n + c];
      else A->vals[row * 27 + found] = v[r * n + c];
    }
  }
  return 0;
}
DM ch_standin_matdm = NULL;
PetscErrorCode MatAssemblyBegin(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatAssemblyEnd(Mat A, MatAssemblyType t) { (void)A; (void)t; return 0; }
PetscErrorCode MatZeroEntries(Mat A) {
  for (int r = 0; r < A->N; ++r)
    for (int q = 0; q < A->ncols[r]; ++q) A->vals[r * 27 + q] = 0.0;
  return 0;
}
PetscErrorCode MatShift(Mat A, PetscScalar a) {
  for (int r = 0; r < A->N; ++r) {
    int q, found = -1;
    for (q = 0; q < A->ncols[r]; ++q)
      if (A->cols[r * 27 + q] == r) { found = q; break; }
    if (found < 0) { found = A->ncols[r]++; A->cols[r * 27 + found] = r; A->vals[r * 27 + found] = 0.0; }
    A->vals[r * 27 + found] += a;
  }
  return 0;
}
PetscErrorCode MatView(Mat A, PetscViewer v) { (void)A; (void)v; return 0; }
PetscErrorCode MatCreateVecs(Mat A, Vec* r, Vec* l) { (void)A; (void)r; (void)l; return PETSC_ERR_ARG_WRONG; }
struct _p_MatNullSpace { int dummy; };
PetscErrorCode MatNullSpaceCreate(MPI_Comm c, PetscBool has_cnst, PetscInt n, const Vec* vecs, MatNullSpace* sp) {
  (void)c; (void)has_cnst; (void)n; (void)vecs;
  *sp = (MatNullSpace)calloc(1, sizeof(**sp));
  return 0;
}
PetscErrorCode MatSetNullSpace(Mat A, MatNullSpace sp) { (void)A; (void)sp; return 0; }
PetscErrorCode MatNullSpaceDestroy(MatNullSpace* sp) { free(*sp); *sp = NULL; return 0; }
PetscErrorCode MatNullSpaceRemove(MatNullSpace sp, Vec v) {
  (void)sp;
  double m;
  VecMean(v, &m);
  for (int i = 0; i < v->n; ++i) v->a[i] -= m;
  return 0;
}
PetscErrorCode KSPGetDM(KSP ksp, DM* dm) { *dm = ksp->dm; return 0; }
PetscErrorCode KSPGetSolution(KSP ksp, Vec* v) { *v = ksp->sol; return 0; }
PetscErrorCode KSPGetOperators(KSP ksp, Mat* A, Mat* P) { if (A) *A = ksp->A; if (P) *P = ksp->A; return 0; }
/* ---------------- options database and KSP settings ---------------- */
#define CH_STANDIN_MAXOPT 64
static char* g_opt_name[CH_STANDIN_MAXOPT];
static char* g_opt_val[CH_STANDIN_MAXOPT];
static int g_nopt = 0;

void ch_standin_options(int argc, const char* const* argv) {
  for (int i = 0; i < g_nopt; ++i) { free(g_opt_name[i]); free(g_opt_val[i]); }
  g_nopt = 0;
  for (int i = 0; i < argc && g_nopt < CH_STANDIN_MAXOPT; ++i) {
    if (argv[i][0] != '-') continue;
    const int has_val = i + 1 < argc && argv[i + 1][0] != '-';
    g_opt_name[g_nopt] = strdup(argv[i]);
    g_opt_val[g_nopt] = has_val ? strdup(argv[i + 1]) : NULL;
    ++g_nopt;
    if (has_val) ++i;
  }
}

static const char* opt_find(const char* name, int* found) {
  *found = 0;
  for (int i = g_nopt - 1; i >= 0; --i)
    if (!strcmp(g_opt_name[i], name)) { *found = 1; return g_opt_val[i]; }
  return NULL;
}

PetscErrorCode PetscOptionsGetString(PetscOptions o, const char pre[], const char name[], char str[], size_t len,
                                     PetscBool* set) {
  (void)o; (void)pre;
  int f;
  const char* v = opt_find(name, &f);
  *set = (f && v) ? PETSC_TRUE : PETSC_FALSE;
  if (*set && len) { strncpy(str, v, len - 1); str[len - 1] = 0; }
  return 0;
}
PetscErrorCode PetscOptionsGetInt(PetscOptions o, const char pre[], const char name[], PetscInt* v, PetscBool* set) {
  (void)o; (void)pre;
  int f;
  const char* s = opt_find(name, &f);
  *set = (f && s) ? PETSC_TRUE : PETSC_FALSE;
  if (*set) *v = (PetscInt)strtol(s, NULL, 10);
  return 0;
}
PetscErrorCode PetscOptionsGetReal(PetscOptions o, const char pre[], const char name[], PetscReal* v,
                                   PetscBool* set) {
  (void)o; (void)pre;
  int f;
  const char* s = opt_find(name, &f);
  *set = (f && s) ? PETSC_TRUE : PETSC_FALSE;
  if (*set) *v = strtod(s, NULL);
  return 0;
}
PetscErrorCode PetscOptionsHasName(PetscOptions o, const char pre[], const char name[], PetscBool* set) {
  (void)o; (void)pre;
  int f;
  (void)opt_find(name, &f);
  *set = f ? PETSC_TRUE : PETSC_FALSE;
  return 0;
}

KSP ch_standin_ksp(DM dm) {
  KSP k = (KSP)calloc(1, sizeof(*k));
  k->dm = dm;
  strcpy(k->type, KSPGMRES);
  k->rtol = 1e-5; k->abstol = 1e-50; k->dtol = 1e4; k->maxits = 10000;
  PetscBool set;
  char buf[32];
  PetscOptionsGetString(NULL, NULL, "-ksp_type", buf, sizeof buf, &set);
  if (set) strcpy(k->type, buf);
  PetscOptionsGetReal(NULL, NULL, "-ksp_rtol", &k->rtol, &set);
  PetscOptionsGetReal(NULL, NULL, "-ksp_atol", &k->abstol, &set);
  PetscOptionsGetInt(NULL, NULL, "-ksp_max_it", &k->maxits, &set);
  return k;
}
PetscErrorCode KSPGetTolerances(KSP ksp, PetscReal* rtol, PetscReal* abstol, PetscReal* dtol, PetscInt* maxits) {
  if (rtol) *rtol = ksp->rtol;
  if (abstol) *abstol = ksp->abstol;
  if (dtol) *dtol = ksp->dtol;
  if (maxits) *maxits = ksp->maxits;
  return 0;
}
PetscErrorCode KSPGetType(KSP ksp, KSPType* type) { *type = ksp->type; return 0; }

PetscErrorCode PetscViewerBinaryOpen(MPI_Comm c, const char* n, PetscFileMode m, PetscViewer* v) {
  (void)c; (void)n; (void)m; *v = NULL;
  return PETSC_ERR_ARG_WRONG;
}
PetscErrorCode PetscViewerDestroy(PetscViewer* v) { (void)v; return 0; }

/* ---------------- SLEPc (never called) ---------------- */
#define NOSLEPC { return PETSC_ERR_ARG_WRONG; }
PetscErrorCode EPSCreate(MPI_Comm c, EPS* e) { (void)c; (void)e; NOSLEPC }
PetscErrorCode EPSSetOperators(EPS e, Mat A, Mat B) { (void)e; (void)A; (void)B; NOSLEPC }
PetscErrorCode EPSSetProblemType(EPS e, EPSProblemType t) { (void)e; (void)t; NOSLEPC }
PetscErrorCode EPSSetFromOptions(EPS e) { (void)e; NOSLEPC }
PetscErrorCode EPSSolve(EPS e) { (void)e; NOSLEPC }
PetscErrorCode EPSGetIterationNumber(EPS e, PetscInt* i) { (void)e; (void)i; NOSLEPC }
PetscErrorCode EPSGetType(EPS e, EPSType* t) { (void)e; (void)t; NOSLEPC }
PetscErrorCode EPSGetDimensions(EPS e, PetscInt* a, PetscInt* b, PetscInt* c) { (void)e; (void)a; (void)b; (void)c; NOSLEPC }
PetscErrorCode EPSGetTolerances(EPS e, PetscReal* t, PetscInt* m) { (void)e; (void)t; (void)m; NOSLEPC }
PetscErrorCode EPSGetConverged(EPS e, PetscInt* n) { (void)e; (void)n; NOSLEPC }
PetscErrorCode EPSGetEigenpair(EPS e, PetscInt i, PetscScalar* a, PetscScalar* b, Vec x, Vec y) {
  (void)e; (void)i; (void)a; (void)b; (void)x; (void)y; NOSLEPC
}
PetscErrorCode EPSComputeError(EPS e, PetscInt i, EPSErrorType t, PetscReal* r) { (void)e; (void)i; (void)t; (void)r; NOSLEPC }
PetscErrorCode EPSDestroy(EPS* e) { (void)e; return 0; }
