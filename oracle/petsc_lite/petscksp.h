/* petsc-lite: forwards to petscsys.h (TEST INFRASTRUCTURE ONLY). */
#include "petscsys.h"
