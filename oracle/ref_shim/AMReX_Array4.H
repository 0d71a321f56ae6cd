// Single-box AMReX stand-in (test infrastructure); see axs_amrex_shim.H.
#pragma once
#include "axs_amrex_shim.H"
