#ifndef KOKKOS_DECLARE_CONFIG_HAND_WRITTEN
#define KOKKOS_DECLARE_CONFIG_HAND_WRITTEN
#include <decl/Kokkos_Declare_OPENMP.hpp>
#include <decl/Kokkos_Declare_SERIAL.hpp>
#endif
