/* Empty stand-in for the reference's CMake-generated SystemConfig.h.
 * Leaving USE_ALIGNED_ALLOCATOR undefined keeps Boost.Align out of the
 * reference's kmeans_common.hpp when oracle/build_ref.sh compiles it. */
