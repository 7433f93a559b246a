/* Hand-written stand-in for the header Kokkos' configure step would write:
 * Kokkos 4.3.1, OpenMP (default) and Serial host back ends, C++20.  Used only
 * to compile the reference's stock main with OpenMP threads for the CPU
 * timing baseline (oracle/ref). */
#if !defined(KOKKOS_MACROS_HPP) || defined(KOKKOS_CORE_CONFIG_H)
#error "Do not include KokkosCore_config.h directly; include Kokkos_Macros.hpp instead."
#else
#define KOKKOS_CORE_CONFIG_H
#endif
#define KOKKOS_VERSION 40301
#define KOKKOS_VERSION_MAJOR 4
#define KOKKOS_VERSION_MINOR 3
#define KOKKOS_VERSION_PATCH 1
#define KOKKOS_ENABLE_OPENMP
#define KOKKOS_ENABLE_SERIAL
#define KOKKOS_ENABLE_CXX20
#define KOKKOS_ENABLE_LIBDL
