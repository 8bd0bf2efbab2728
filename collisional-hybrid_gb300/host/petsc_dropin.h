/*
 * petsc_dropin.h -- helpers of the GPU drop-in (petsc_dropin.c) for a PETSc
 * host that edits the ions itself between the hot-path calls.  The
 * reference's own loop (src/hybrid.c:101-123) needs neither.
 */
#ifndef CH_PETSC_DROPIN_H
#define CH_PETSC_DROPIN_H
#include <petsc.h>

#include "hybrid.h"

/* The host changed the DMSwarm "position"/"velocity" fields in place: the
 * next particle call uploads them. */
PetscErrorCode HybridGPUIonsChanged(void);
/* Copies the device's ions into the DMSwarm fields if the device holds
 * newer ones (after UpdateVelocities, before UpdatePositions). */
PetscErrorCode HybridGPUSyncIons(Context* ctx);
#endif
