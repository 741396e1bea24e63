/* Read access to the stand-in's dense storage, for the oracle's dump driver. */
#ifndef TDBEM_REF_SHIM_ACCESS_H
#define TDBEM_REF_SHIM_ACCESS_H
#include "petscsys.h"
const double* shim_mat_data(Mat A, int* m, int* n);
const double* shim_vec_data(Vec v, int* n);
#endif
