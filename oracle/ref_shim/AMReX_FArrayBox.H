// Stand-in header for the oracle build of the reference sources (test infrastructure only).
#pragma once
#include "amrex_shim.H"
