/* shim: see petsc_shim.h */
#include "petsc_shim.h"
