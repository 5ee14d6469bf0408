// Version header for the oracle's build of the reference templates (test infrastructure);
// stands in for the one the reference's CMake generates from utopia/utopia_Version.hpp.in.
#ifndef UTOPIA_VERSION_HPP
#define UTOPIA_VERSION_HPP
#define UTOPIA_VERSION_MAJOR 0
#define UTOPIA_VERSION_MINOR 0
#define UTOPIA_VERSION_PATCH 0
#define UTOPIA_GIT_VERSION "unknown"
#define UTOPIA_VERSION "0.0.0"
#endif  // UTOPIA_VERSION_HPP
