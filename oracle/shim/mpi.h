/* ORACLE shim: the reference's base definitions include <mpi.h>
 * (Definitions.cpp:69-70); the hot path makes no MPI call, so nothing is declared. */
#pragma once
