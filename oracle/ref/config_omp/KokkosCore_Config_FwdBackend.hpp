#ifndef KOKKOS_FWD_CONFIG_HAND_WRITTEN
#define KOKKOS_FWD_CONFIG_HAND_WRITTEN
#include <fwd/Kokkos_Fwd_OPENMP.hpp>
#include <fwd/Kokkos_Fwd_SERIAL.hpp>
#endif
