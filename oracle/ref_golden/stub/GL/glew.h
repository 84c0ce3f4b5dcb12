/* Compile-only declarations so that the reference's tsdf.cuh/tsdf.cu, which
 * include GL headers for GpuTsdfGenerator::render, build without a graphics
 * stack.  render() is never called; nothing here draws or loads a library. */
#pragma once
#define GL_TRIANGLES 0x0004
static inline void glBegin(int) {}
static inline void glEnd(void) {}
static inline void glColor3f(float, float, float) {}
static inline void glVertex3f(float, float, float) {}
