// Stand-in for the reference's shaders/common/common.glsl when its render
// shaders are compiled as C++ (TEST INFRASTRUCTURE ONLY).  The vertex shaders
// open with #include "common/common.glsl"; this directory comes first on the
// include path, so that line lands here.  What the shaders take from that file
// (types, uniforms, relativeLocation, emptyAABB) is restated in
// render_shim.hpp, which ref_render.cpp includes before the shaders.
