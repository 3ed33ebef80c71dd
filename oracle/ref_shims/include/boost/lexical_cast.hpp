// Empty stand-in: industry3d/src/utility.cpp includes this Boost header but
// uses nothing from it, so the file compiles without Boost.  Test
// infrastructure only.
#pragma once
