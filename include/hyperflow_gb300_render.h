/* HyperFlow-GB300 -- frame images on the GPU (the reference's offline plotting script,
 * src/visualisation/euler/euler_2d.py, headless).
 *
 * The reference pivots each CSV frame onto the domain's cell grid and shows one flow variable
 * (rho, u, v, p) or its "schlieren-like" normalised exponentiated gradient
 * (euler_2d.py:214-295: central differences over the interior cells, s = beta * exp(-lambda *
 * |grad| / max |grad|), beta 1, lambda 15, the boundary cells' gradient 0) with matplotlib's
 * imshow.  Here a kernel forms the same field and an 8-bit grey image from a domain grid in
 * device memory; hyperflow_gb300/render.py assembles the grid from binary frames and writes PNG
 * files.  Status codes are the HF_* codes of hyperflow_gb300.h.
 */
#ifndef HYPERFLOW_GB300_RENDER_H
#define HYPERFLOW_GB300_RENDER_H

#include "hyperflow_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

/* d_field: device array [ny][nx] (x fastest; NaN where no block covers the domain), cell sizes
 * dx, dy.  schlieren = 1 forms the gradient field above into d_out (device, nx * ny doubles;
 * required then, optional otherwise) and images it; 0 images d_field itself.  limits (host, two
 * doubles, or NULL for the finite minimum and maximum of the imaged field) map linearly onto grey
 * levels 0..255, rounded; NaN cells are 0.  d_image: device [ny][nx] bytes, row 0 at the bottom
 * (y up, as imshow's origin='lower').  Asynchronous on stream (a cudaStream_t, NULL for the
 * default stream).  Calls that overlap on the GPU share a small static reduction area. */
int hf_render_gray(const double* d_field, int nx, int ny, double dx, double dy, int schlieren, double beta,
                   double lambda, const double* limits, double* d_out, unsigned char* d_image, void* stream);

#ifdef __cplusplus
}
#endif
#endif
