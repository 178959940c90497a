// Drop-in C++ layer over librast for canmom/rasteriser.
//
// rast_dropin.cpp defines, with the reference's exact signatures, every function its headers
// declare on the per-frame path:
//   geometry.h:14-40  transformation_matrix, camera_matrix, transform_direction, transform_point,
//                     z_divide, remap_ndc, ndc_to_raster, signed_area_2d, transform_vertices,
//                     transform_normals, z_divide_all, xyz_all, transform_lights,
//                     ndc_to_raster_all, and Light::transform (light.h:13)
//   drawing.h:16-18   draw_frame  -> one rast_draw on the GPU
//   shading.h:10-12   light_contribution, shade
// Linking rast_dropin.o and librast.so in place of the reference's geometry.o, drawing.o and
// shading.o leaves renderer.cpp, arguments.cpp, fileloader.cpp and material.cpp unchanged.
//
// This header adds the few controls the reference does not have. Include it only where they are
// wanted; the drop-in works without it.
#ifndef RAST_DROPIN_H
#define RAST_DROPIN_H

namespace rast_dropin {

// Projection used by camera_matrix. The reference fixes 45 degrees, near 0.1, far 6
// (geometry.cpp:30), which is the default here.
void set_projection(float fovy_degrees, float z_near, float z_far);

// CUDA device of the process-wide context (default 0, or the RAST_DEVICE environment variable).
// Takes effect before the first draw_frame.
void set_device(int device);

// draw_frame re-uploads the mesh on every call by default, because the reference's const vectors
// may change between calls. A caller that draws the same, unmodified vectors frame after frame (the
// spin loop, renderer.cpp:104-125) can declare them static: the mesh is then uploaded again only
// when a vector's address or size changes.
void set_static_mesh(bool is_static);

// Releases the process-wide context.
void shutdown();

}  // namespace rast_dropin

#endif
