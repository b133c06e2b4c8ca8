// Oracle build support: the parallel-for algorithms live in taskflow.hpp's
// stand-in (tf::Taskflow::for_each_index).
#pragma once
#include "../taskflow.hpp"
