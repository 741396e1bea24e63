/* Mat declarations live in petscsys.h of this single-rank stand-in. */
#ifndef TDBEM_REF_SHIM_PETSCMAT_H
#define TDBEM_REF_SHIM_PETSCMAT_H
#include "petscsys.h"
#endif
