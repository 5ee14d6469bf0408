// Configuration header for compiling the reference's solver templates as the oracle's pin
// (test infrastructure).  It stands in for the header the reference's CMake generates from
// utopia/utopia_Config.hpp.in: no optional backend or dependency is enabled (no MPI, PETSc,
// Trilinos, BLAS, YAML, tracing), lambdas are host lambdas and lock checks are off.
#ifndef UTOPIA_CONFIG_HPP
#define UTOPIA_CONFIG_HPP

#define UTOPIA_CXX_COMPILER "g++"
#define UTOPIA_C_COMPILER "gcc"
#define UTOPIA_DEP_INCLUDES ""
#define UTOPIA_DEP_LIBRARIES ""

#define UTOPIA_ENABLE_CPP14
#define UTOPIA_ENABLE_CPP17

#define UTOPIA_LAMBDA [=]
#define UTOPIA_INLINE_FUNCTION inline
#define UTOPIA_INLINE_FUNCTION_DEFAULTED inline
#define UTOPIA_FUNCTION
#define UTOPIA_NVCC_PRIVATE

#define utopia_lock_check_assert(expr_)

#define UTOPIA_DEPRECATED __attribute__((__deprecated__))
#define UTOPIA_DEPRECATED_MSG(MSG) __attribute__((__deprecated__(MSG)))

#endif  // UTOPIA_CONFIG_HPP
