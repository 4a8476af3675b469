/* forwards to the PETSc type stand-in (oracle only) */
#include "petsc.h"
