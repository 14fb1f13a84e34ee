// Test infrastructure only (oracle build of the reference). Replacement for the
// reference's precompiled header src/stdafx.h: the same standard headers,
// OpenMP and tinyformat, but none of boost::asio/filesystem, OpenGL, GLFW or
// OpenCL, which are absent here and are not needed by the CPU hot path.
#pragma once

#include <algorithm>
#include <array>
#include <atomic>
#include <cassert>
#include <chrono>
#include <cmath>
#include <complex>
#include <cstddef>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <ctime>
#include <fstream>
#include <functional>
#include <iostream>
#include <limits>
#include <map>
#include <mutex>
#include <numeric>
#include <random>
#include <regex>
#include <stdexcept>
#include <string>
#include <sstream>
#include <thread>
#include <vector>

#include <omp.h>
#include <errno.h>
#include <stdlib.h>
#include <sys/types.h>
#include <unistd.h>

#include <boost/align/aligned_allocator.hpp>

#include "tinyformat/tinyformat.h"
#include "Common.h"
