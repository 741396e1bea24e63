/* KSP declarations live in petscsys.h of this single-rank stand-in. */
#ifndef TDBEM_REF_SHIM_PETSCKSP_H
#define TDBEM_REF_SHIM_PETSCKSP_H
#include "petscsys.h"
#endif
