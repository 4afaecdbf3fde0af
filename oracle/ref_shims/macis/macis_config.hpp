// Generated-config stand-in for the reference's CMake-configured header:
// MPI is disabled (single-process build of the reference's headers).
#pragma once
