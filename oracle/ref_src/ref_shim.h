/*
 * Pre-include for compiling the reference's headers into the golden-vector
 * generator on the build host (TEST INFRASTRUCTURE ONLY).  The standard headers are pulled in
 * first so that "#define private public" below touches no library header;
 * the reference's evaluator classes keep their tables and vectors private,
 * and the golden-vector generator reads and sets them directly.
 */
#include <algorithm>
#include <array>
#include <chrono>
#include <cmath>
#include <cstdlib>
#include <cstring>
#include <iomanip>
#include <iostream>
#include <limits>
#include <memory>
#include <string>
#include <vector>
#include <sys/time.h>
#ifdef _OPENMP
#include <omp.h>
#endif
#define private public
