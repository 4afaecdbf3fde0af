// Generated-config stand-in for sparsexx's CMake-configured header: no MPI,
// no optional backends.
#pragma once
