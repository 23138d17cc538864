/* Empty stand-in for the reference's src/glvu/glvu.h so that the reference's
   FLUID_3D_MIC.cpp (which includes it through BOX.h / OBSTACLE.h) compiles
   without OpenGL.  The oracle never draws.  TEST INFRASTRUCTURE ONLY. */
#ifndef PLUME_ORACLE_GLVU_SHIM_H
#define PLUME_ORACLE_GLVU_SHIM_H
#endif
