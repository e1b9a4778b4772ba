#pragma once
// Part of the host-only Kokkos shim used to build the reference oracle.
#include "Kokkos_Core.hpp"
