// Stand-in for the CMake-generated configuration header.
#pragma once
#define OMPL_VERSION "oracle"
#define OMPL_MAJOR_VERSION 2
#define OMPL_MINOR_VERSION 0
#define OMPL_PATCH_VERSION 0
#define OMPL_VERSION_VALUE 2000000
#define OMPL_HAVE_FLANN 0
#define OMPL_HAVE_SPOT 0
#define OMPL_HAVE_NUMPY 0
