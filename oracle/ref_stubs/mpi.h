/* No MPI in this image; the single-GPU build of the reference (USE_MPI=0)
 * includes <mpi.h> but uses none of its symbols in the CPU parts built here. */
#pragma once
