/* GraphCut.cu -- the name the reference's callers include
 * (solveMRF.cu:67, Application.cu:5, Debug.cu:5).  Everything is in
 * GraphCut.h, a C++ front end of the gcfg shared library; this file holds no
 * code of its own. */
#include "GraphCut.h"
