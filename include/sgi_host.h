/*
 * sgi_host.h - host-side preparation of the frame's VPL buffer (no device work).
 *
 * Replaces the VPL branch of RendererBackend::UpdatePointLights_
 * (Source/Engine/StratusRendererBackend.cpp:1357-1389) and InitVplFrameData_
 * (:1281-1292): the VPLs whose bounding sphere touches the view frustum
 * (IsSphereInFrustum, Source/Engine/StratusMath.h:401-412) are ordered by
 * their distance to the camera (a std::multiset of VplDistKey_, so equal
 * distances keep the input order), the first `cap` are kept (the reference:
 * MAX_TOTAL_VPLS_BEFORE_CULLING = 10000) and packed as GpuVplData records
 * with position (x, y, z, 1), radius, far plane and intensity; colour and
 * specular position stay zero until the VPL colouring pass fills them
 * (sgi_set_vpl_coloring).
 *
 * Arithmetic, in binary32 with each operation rounded on its own:
 *   distance = sqrt((dx*dx + dy*dy) + dz*dz), d = position - camera
 *   (glm::distance), and a sphere is outside when for some plane
 *   (a*x + b*y) + (c*z + d*1) < -radius: the four products added in pairs,
 *   as glm::dot of two vec4 adds them (glm/detail/func_geometric.inl:64-70).
 *
 * Non-finite planes, camera, positions or radii return SGI_ERR_ARG (a NaN
 * distance has no place in the distance order).
 */
#ifndef SGI_HOST_H_
#define SGI_HOST_H_

#include "sgi.h"

#ifdef __cplusplus
extern "C" {
#endif

/* positions [n][3], radii / far_planes / intensities [n], planes [6][4]
 * (the frame's view-frustum planes, inward normals), camera [3].
 * out [min(n, cap)] receives the kept VPLs in distance order, source
 * [min(n, cap)] (optional) their input indices, *count how many were kept. */
sgi_status sgi_prepare_vpls(const float* positions, const float* radii, const float* far_planes,
                            const float* intensities, int32_t n, const float* planes, const float* camera,
                            int32_t cap, sgi_vpl* out, int32_t* source, int32_t* count);

#ifdef __cplusplus
}
#endif

#endif /* SGI_HOST_H_ */
