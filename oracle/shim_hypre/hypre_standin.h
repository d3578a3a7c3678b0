/* Test infrastructure: a stand-in for the part of Hypre's public SStruct /
 * ParCSR interface that the reference's environment.c calls, so that file can
 * be compiled unmodified and run at one rank without Hypre (which is neither
 * vendored nor installed).  The stand-in stores the assembled system node by
 * node (one part, box order: x fastest) and solves it with its own conjugate
 * gradients; it exports readers for the assembled matrix and vectors.  Only
 * the names and argument meanings follow Hypre's documented interface. */
#ifndef TM_HYPRE_STANDIN_H
#define TM_HYPRE_STANDIN_H

/* Hypre's utilities header brings in the C library's I/O and allocation
 * declarations, which environment.c relies on */
#include <stdio.h>
#include <stdlib.h>

#include "mpi.h"

typedef int HYPRE_Int;
typedef double HYPRE_Real;
typedef double HYPRE_Complex;

typedef enum {
    HYPRE_SSTRUCT_VARIABLE_UNDEFINED = -1,
    HYPRE_SSTRUCT_VARIABLE_CELL = 0,
    HYPRE_SSTRUCT_VARIABLE_NODE = 1
} HYPRE_SStructVariable;

#define HYPRE_PARCSR 5555

typedef struct hs_grid *HYPRE_SStructGrid;
typedef struct hs_stencil *HYPRE_SStructStencil;
typedef struct hs_graph *HYPRE_SStructGraph;
typedef struct hs_matrix *HYPRE_SStructMatrix;
typedef struct hs_vector *HYPRE_SStructVector;
typedef struct hs_matrix *HYPRE_ParCSRMatrix;
typedef struct hs_vector *HYPRE_ParVector;
typedef struct hs_solver *HYPRE_Solver;
typedef HYPRE_Int (*HYPRE_PtrToParSolverFcn)(HYPRE_Solver, HYPRE_ParCSRMatrix, HYPRE_ParVector, HYPRE_ParVector);

HYPRE_Int HYPRE_SStructGridCreate(MPI_Comm comm, HYPRE_Int ndim, HYPRE_Int nparts, HYPRE_SStructGrid *grid);
HYPRE_Int HYPRE_SStructGridSetExtents(HYPRE_SStructGrid grid, HYPRE_Int part, HYPRE_Int *ilower, HYPRE_Int *iupper);
HYPRE_Int HYPRE_SStructGridSetVariables(HYPRE_SStructGrid grid, HYPRE_Int part, HYPRE_Int nvars,
                                        HYPRE_SStructVariable *vartypes);
HYPRE_Int HYPRE_SStructGridAssemble(HYPRE_SStructGrid grid);

HYPRE_Int HYPRE_SStructStencilCreate(HYPRE_Int ndim, HYPRE_Int size, HYPRE_SStructStencil *stencil);
HYPRE_Int HYPRE_SStructStencilSetEntry(HYPRE_SStructStencil stencil, HYPRE_Int entry, HYPRE_Int *offset,
                                       HYPRE_Int var);

HYPRE_Int HYPRE_SStructGraphCreate(MPI_Comm comm, HYPRE_SStructGrid grid, HYPRE_SStructGraph *graph);
HYPRE_Int HYPRE_SStructGraphSetObjectType(HYPRE_SStructGraph graph, HYPRE_Int type);
HYPRE_Int HYPRE_SStructGraphSetStencil(HYPRE_SStructGraph graph, HYPRE_Int part, HYPRE_Int var,
                                       HYPRE_SStructStencil stencil);
HYPRE_Int HYPRE_SStructGraphAssemble(HYPRE_SStructGraph graph);

HYPRE_Int HYPRE_SStructMatrixCreate(MPI_Comm comm, HYPRE_SStructGraph graph, HYPRE_SStructMatrix *matrix);
HYPRE_Int HYPRE_SStructMatrixSetObjectType(HYPRE_SStructMatrix matrix, HYPRE_Int type);
HYPRE_Int HYPRE_SStructMatrixInitialize(HYPRE_SStructMatrix matrix);
HYPRE_Int HYPRE_SStructMatrixSetBoxValues(HYPRE_SStructMatrix matrix, HYPRE_Int part, HYPRE_Int *ilower,
                                          HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Int nentries, HYPRE_Int *entries,
                                          HYPRE_Complex *values);
HYPRE_Int HYPRE_SStructMatrixAddToBoxValues(HYPRE_SStructMatrix matrix, HYPRE_Int part, HYPRE_Int *ilower,
                                            HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Int nentries,
                                            HYPRE_Int *entries, HYPRE_Complex *values);
HYPRE_Int HYPRE_SStructMatrixAssemble(HYPRE_SStructMatrix matrix);
HYPRE_Int HYPRE_SStructMatrixGetObject(HYPRE_SStructMatrix matrix, void **object);

HYPRE_Int HYPRE_SStructVectorCreate(MPI_Comm comm, HYPRE_SStructGrid grid, HYPRE_SStructVector *vector);
HYPRE_Int HYPRE_SStructVectorSetObjectType(HYPRE_SStructVector vector, HYPRE_Int type);
HYPRE_Int HYPRE_SStructVectorInitialize(HYPRE_SStructVector vector);
HYPRE_Int HYPRE_SStructVectorSetBoxValues(HYPRE_SStructVector vector, HYPRE_Int part, HYPRE_Int *ilower,
                                          HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Complex *values);
HYPRE_Int HYPRE_SStructVectorAddToBoxValues(HYPRE_SStructVector vector, HYPRE_Int part, HYPRE_Int *ilower,
                                            HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Complex *values);
HYPRE_Int HYPRE_SStructVectorGetBoxValues(HYPRE_SStructVector vector, HYPRE_Int part, HYPRE_Int *ilower,
                                          HYPRE_Int *iupper, HYPRE_Int var, HYPRE_Complex *values);
HYPRE_Int HYPRE_SStructVectorAssemble(HYPRE_SStructVector vector);
HYPRE_Int HYPRE_SStructVectorGather(HYPRE_SStructVector vector);
HYPRE_Int HYPRE_SStructVectorGetObject(HYPRE_SStructVector vector, void **object);

HYPRE_Int HYPRE_ParCSRPCGCreate(MPI_Comm comm, HYPRE_Solver *solver);
HYPRE_Int HYPRE_ParCSRPCGSetTol(HYPRE_Solver solver, HYPRE_Real tol);
HYPRE_Int HYPRE_ParCSRPCGSetPrintLevel(HYPRE_Solver solver, HYPRE_Int level);
HYPRE_Int HYPRE_ParCSRPCGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter);
HYPRE_Int HYPRE_ParCSRPCGSetPrecond(HYPRE_Solver solver, HYPRE_PtrToParSolverFcn precond,
                                    HYPRE_PtrToParSolverFcn precond_setup, HYPRE_Solver precond_solver);
HYPRE_Int HYPRE_ParCSRPCGSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x);
HYPRE_Int HYPRE_ParCSRPCGSolve(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x);

HYPRE_Int HYPRE_BoomerAMGCreate(HYPRE_Solver *solver);
HYPRE_Int HYPRE_BoomerAMGSetMaxIter(HYPRE_Solver solver, HYPRE_Int max_iter);
HYPRE_Int HYPRE_BoomerAMGSetTol(HYPRE_Solver solver, HYPRE_Real tol);
HYPRE_Int HYPRE_BoomerAMGSetPrintLevel(HYPRE_Solver solver, HYPRE_Int level);
HYPRE_Int HYPRE_BoomerAMGSetCoarsenType(HYPRE_Solver solver, HYPRE_Int type);
HYPRE_Int HYPRE_BoomerAMGSetRelaxType(HYPRE_Solver solver, HYPRE_Int type);
HYPRE_Int HYPRE_BoomerAMGSetNumSweeps(HYPRE_Solver solver, HYPRE_Int sweeps);
HYPRE_Int HYPRE_BoomerAMGSetup(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x);
HYPRE_Int HYPRE_BoomerAMGSolve(HYPRE_Solver solver, HYPRE_ParCSRMatrix A, HYPRE_ParVector b, HYPRE_ParVector x);

#endif
