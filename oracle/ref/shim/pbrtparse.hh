/* pbrtlex.cpp includes "pbrtparse.hh"; the fork ships the generated header
 * as core/pbrtparse.hpp. */
#include "pbrtparse.hpp"
