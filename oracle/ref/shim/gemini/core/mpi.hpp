/*
 * Test-only stand-in for the two GeminiGraph helpers that
 * include/mpi_helper.hpp:30-32 pulls in: get_mpi_data_type<T>() and
 * MPI_Instance.  With the single-rank shim in ../../mpi.h a datatype is the
 * element size in bytes.  Oracle infrastructure only.
 */
#pragma once

#include "mpi.h"

template <typename T>
inline MPI_Datatype get_mpi_data_type()
{
    return sizeof(T);
}

class MPI_Instance
{
public:
    MPI_Instance(int *, char ***) {}
};
