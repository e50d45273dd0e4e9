// Declarations of the cairo calls the reference's visualiser makes
// (Visualizer.cpp), so that it compiles without cairo; oracle/ref_placer.cpp
// defines them as no-ops.  TEST INFRASTRUCTURE ONLY.
#pragma once
typedef struct _cairo_surface cairo_surface_t;
typedef struct _cairo cairo_t;
typedef enum { CAIRO_FORMAT_ARGB32 = 0, CAIRO_FORMAT_RGB24 = 1 } cairo_format_t;
#ifdef __cplusplus
extern "C" {
#endif
cairo_surface_t *cairo_image_surface_create(cairo_format_t, int, int);
cairo_t *cairo_create(cairo_surface_t *);
void cairo_scale(cairo_t *, double, double);
void cairo_rectangle(cairo_t *, double, double, double, double);
void cairo_set_source_rgb(cairo_t *, double, double, double);
void cairo_paint(cairo_t *);
void cairo_set_line_width(cairo_t *, double);
void cairo_stroke(cairo_t *);
void cairo_fill(cairo_t *);
int cairo_surface_write_to_png(cairo_surface_t *, const char *);
#ifdef __cplusplus
}
#endif
