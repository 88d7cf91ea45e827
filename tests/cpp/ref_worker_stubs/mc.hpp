// Stand-in for the reference's src/mc.hpp when the reference's own
// gpuWorker.cpp / gpuWorker.hpp are compiled against the drop-in: the class
// `mc` comes from include/gpda_mc.hpp. TEST INFRASTRUCTURE ONLY.
#pragma once
#include <string>
#include <vector>
using namespace std;   // the reference's mc.hpp opens namespace std for its includers
#include "gpda_mc.hpp"
