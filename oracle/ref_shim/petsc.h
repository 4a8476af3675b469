/* PETSc *type* stand-in used only to compile the reference's element,
 * material, shape and Gauss-point translation units for the CPU oracle
 * (oracle/_ref). It declares the handful of PETSc types and the four
 * insertion / printing calls those units reference; none of them does any
 * linear algebra. Complex build, as elpasoC is built with PETSC_USE_COMPLEX.
 * This is test infrastructure, not product code. */
#pragma once
#include <complex>
#include <cstdio>
#include <cstdarg>
#include <cmath>
typedef int PetscInt;
typedef int PetscMPIInt;
typedef double PetscReal;
typedef std::complex<double> PetscScalar;
typedef std::complex<double> PetscComplex;
typedef double PetscLogDouble;
typedef int PetscErrorCode;
typedef enum { PETSC_FALSE = 0, PETSC_TRUE = 1 } PetscBool;
typedef enum { NOT_SET_VALUES, INSERT_VALUES, ADD_VALUES } InsertMode;
struct _p_Mat; typedef _p_Mat* Mat;
struct _p_Vec; typedef _p_Vec* Vec;
struct _p_KSP; typedef _p_KSP* KSP;
struct _p_PC; typedef _p_PC* PC;
struct _p_AO; typedef _p_AO* AO;
struct _p_IS; typedef _p_IS* IS;
struct _p_Viewer; typedef _p_Viewer* PetscViewer;
typedef int MPI_Comm;
#define PETSC_COMM_WORLD 0
#define PETSC_COMM_SELF 0
#define PETSC_NULL 0
#ifndef PETSC_USE_COMPLEX
#define PETSC_USE_COMPLEX 1
#endif
#define PETSC_i PetscScalar(0.0, 1.0)
inline PetscReal PetscRealPart(PetscScalar a) { return a.real(); }
inline PetscReal PetscImaginaryPart(PetscScalar a) { return a.imag(); }
inline PetscReal PetscAbsScalar(PetscScalar a) { return std::abs(a); }
inline PetscScalar PetscConj(PetscScalar a) { return std::conj(a); }
/* real PETSc complex builds provide integer x complex products */
inline PetscScalar operator*(int a, const PetscScalar& b) { return PetscScalar((double)a) * b; }
inline PetscScalar operator*(const PetscScalar& b, int a) { return PetscScalar((double)a) * b; }
PetscErrorCode PetscPrintf(MPI_Comm, const char*, ...);
PetscErrorCode PetscFPrintf(MPI_Comm, FILE*, const char*, ...);
PetscErrorCode PetscTime(PetscLogDouble*);
PetscErrorCode MatSetValues(Mat, PetscInt, const PetscInt*, PetscInt, const PetscInt*,
                            const PetscScalar*, InsertMode);
PetscErrorCode VecSetValues(Vec, PetscInt, const PetscInt*, const PetscScalar*, InsertMode);
PetscErrorCode VecSetValue(Vec, PetscInt, PetscScalar, InsertMode);
PetscErrorCode VecGetValues(Vec, PetscInt, const PetscInt*, PetscScalar*);
