// Project-written stand-in for the one Boost.Predef fact the reference's
// cache reader needs (reference include/cache_manager.hpp:4,9-18): which
// operating system the code is compiled for.  Only the *_AVAILABLE macros
// used there are provided.
#ifndef GBBLAS_COMPAT_BOOST_PREDEF_H
#define GBBLAS_COMPAT_BOOST_PREDEF_H

#if defined(__APPLE__) && defined(__MACH__)
#define BOOST_OS_MACOS_AVAILABLE
#elif defined(__linux__)
#define BOOST_OS_LINUX_AVAILABLE
#elif defined(_WIN32)
#define BOOST_OS_WINDOWS_AVAILABLE
#endif

#endif  // GBBLAS_COMPAT_BOOST_PREDEF_H
