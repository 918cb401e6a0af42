/* DataTerm.h -- source-compatible C++ front end of the gcfg_dt_* functions
 * for programs written against the reference's DataTerm namespace
 * (DataTerm.h:9-19, DataTerm.cpp:12-165).
 *
 * Same names and call order as the reference: one process-wide state made by
 * init_data_term(w, h); setImage() with a host image of 3*w*h bytes;
 * selections by selectOnMap() (a 5x5 square, foreground) or setSelection()
 * (host int map: 0 none, 1 foreground, 2 background); getDataTermsMixture()
 * computes the device t-link arrays that getPos()/getNeg() return and that
 * go straight into GC_Init.  The colour model is the 16^3 histogram pair of
 * the selected pixels of the current image; useKernelDensity() switches to
 * the reference's own model (a Gaussian kernel density, whose width
 * setSigmaGaussian() sets; it has no effect on the histogram model).
 * selectBackgroundOnMap() (no counterpart) marks a background square.
 * Errors: a message on stderr and exit(), like the reference's cutil checks.
 * Requires C++17 (inline variables). */
#ifndef GCFG_DATATERM_H_
#define GCFG_DATATERM_H_

#include <cstdio>
#include <cstdlib>

#include "gcfg.h"

namespace DataTerm {

namespace detail {
inline gcfg_dataterm *&state() {
    static gcfg_dataterm *s = NULL;
    return s;
}
inline void check(gcfg_status s, const char *what) {
    if (s != GCFG_OK) {
        fprintf(stderr, "DataTerm::%s failed: %s\n", what, gcfg_strerror(s));
        exit(EXIT_FAILURE);
    }
}
inline gcfg_dataterm *live(const char *what) {
    if (!state()) check(GCFG_ERR_STATE, what);
    return state();
}
}  // namespace detail

/* size of the image and the device arrays, as the reference's globals
 * (DataTerm.h:22-31); valid after init_data_term */
inline int width = 0;
inline int height = 0;
inline unsigned char *d_selection_map = NULL;
inline unsigned char *d_img = NULL;
inline int *d_pos = NULL;
inline int *d_neg = NULL;

inline int *getPos() { return gcfg_dt_pos(detail::live("getPos")); }
inline int *getNeg() { return gcfg_dt_neg(detail::live("getNeg")); }

inline void init_data_term(int w, int h) {
    if (detail::state()) gcfg_dt_destroy(detail::state());
    detail::state() = NULL;
    detail::check(gcfg_dt_create(w, h, &detail::state()), "init_data_term");
    width = w;
    height = h;
    d_selection_map = gcfg_dt_selection(detail::state());
    d_img = gcfg_dt_image(detail::state());
    d_pos = gcfg_dt_pos(detail::state());
    d_neg = gcfg_dt_neg(detail::state());
}

inline void free_data_term() {
    detail::check(gcfg_dt_destroy(detail::live("free_data_term")), "free_data_term");
    detail::state() = NULL;
    d_selection_map = d_img = NULL;
    d_pos = d_neg = NULL;
}

inline void setImage(unsigned char *h_img) {
    detail::check(gcfg_dt_set_image(detail::live("setImage"), h_img), "setImage");
}

inline void setSelection(int *h_select) {
    detail::check(gcfg_dt_set_selection(detail::live("setSelection"), h_select), "setSelection");
}

inline void reset() { detail::check(gcfg_dt_reset(detail::live("reset")), "reset"); }

inline void selectOnMap(int x, int y, int sigma) {
    (void)sigma; /* unused by the reference too (DataTerm.cpp:105-127) */
    detail::check(gcfg_dt_select_on_map(detail::live("selectOnMap"), x, y, 1), "selectOnMap");
}

inline void selectBackgroundOnMap(int x, int y) {
    detail::check(gcfg_dt_select_on_map(detail::live("selectBackgroundOnMap"), x, y, 2), "selectBackgroundOnMap");
}

inline void drawSelection(unsigned char *inp, unsigned char *out) {
    detail::check(gcfg_dt_draw_selection(detail::live("drawSelection"), inp, out), "drawSelection");
}

inline void getDataTermsMixture() {
    detail::check(gcfg_dt_compute(detail::live("getDataTermsMixture")), "getDataTermsMixture");
}

inline void setSigmaGaussian(int sigma) {
    detail::check(gcfg_dt_set_sigma(detail::live("setSigmaGaussian"), sigma), "setSigmaGaussian");
}

/* The reference's own colour model (a kernel density that selectOnMap
 * splats into, DataTerm.cpp:97-137) instead of the histogram pair; call after
 * init_data_term (no counterpart: the reference has only this model). */
inline void useKernelDensity(bool on = true) {
    detail::check(gcfg_dt_set_model(detail::live("useKernelDensity"), on ? GCFG_DT_KDE : GCFG_DT_HISTOGRAM),
                  "useKernelDensity");
}

}  // namespace DataTerm

#endif /* GCFG_DATATERM_H_ */
