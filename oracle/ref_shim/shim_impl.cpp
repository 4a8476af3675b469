/* Test infrastructure (CPU oracle), not product code.
 * Definitions for the PETSc calls and the logging class that the reference
 * element translation units reference. Insertion calls are no-ops: the
 * driver reads element matrices directly. Logging is silenced, as the
 * reference's own test build does with ELPASO_TEST
 * (elpasoCore/source/misc/log/logging.cpp:39-58). */
#include "petsc.h"
#include "misc/log/logging.h"

PetscErrorCode PetscPrintf(MPI_Comm, const char*, ...) { return 0; }
PetscErrorCode PetscFPrintf(MPI_Comm, FILE*, const char*, ...) { return 0; }
PetscErrorCode PetscTime(PetscLogDouble* t) { *t = 0; return 0; }
PetscErrorCode MatSetValues(Mat, PetscInt, const PetscInt*, PetscInt, const PetscInt*,
                            const PetscScalar*, InsertMode) { return 0; }
PetscErrorCode VecSetValues(Vec, PetscInt, const PetscInt*, const PetscScalar*, InsertMode) { return 0; }
PetscErrorCode VecSetValue(Vec, PetscInt, PetscScalar, InsertMode) { return 0; }
PetscErrorCode VecGetValues(Vec, PetscInt, const PetscInt*, PetscScalar*) { return 0; }

FILE* cLogging::logfile = nullptr;
cLogging::cLogging() {}
cLogging::~cLogging() {}
void cLogging::trace(const char[]) {}
void cLogging::message(const char[], ...) {}
void cLogging::openLogFile(const std::string&) {}
void cLogging::closeLogFile() {}
void cLogging::writeDurations(void) {}
