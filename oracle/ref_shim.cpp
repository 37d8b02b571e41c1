// C entry points over the reference's own union-find labelling (ConnComponents.cpp from the
// reference project, compiled unmodified from its source tree by oracle/build_ref.sh).
// TEST INFRASTRUCTURE ONLY: it pins the oracle's labelling restatement; nothing in the
// product links it.
#include <cstdint>
#include <cstdlib>

#include "ConnComponents.h"

extern "C" {

// ConnComponents::label (ConnComponents.cpp:52-86).
void ref_cc_label(unsigned char* img, int w, int h, int* label, int bgval, int conn) {
  nscale::ConnComponents cc;
  cc.label(img, w, h, label, bgval, conn);
}

// ConnComponents::relabel (ConnComponents.cpp:89-118).
int ref_cc_relabel(int w, int h, int* label, int bgval) {
  nscale::ConnComponents cc;
  return cc.relabel(w, h, label, bgval);
}

// ConnComponents::areaThresholdLabeled (ConnComponents.cpp:205-239).
int ref_cc_area_threshold_labeled(const int* label, int w, int h, int* out, int bgval, int lo, int hi) {
  nscale::ConnComponents cc;
  return cc.areaThresholdLabeled(label, w, h, out, bgval, lo, hi);
}

// ConnComponents::areaThreshold (ConnComponents.cpp:150-202).
int ref_cc_area_threshold(unsigned char* img, int w, int h, int* label, int bgval, int lo, int hi, int conn) {
  nscale::ConnComponents cc;
  return cc.areaThreshold(img, w, h, label, bgval, lo, hi, conn);
}

// ConnComponents::boundingBox (ConnComponents.cpp:241-284): copies min(count, cap) entries into
// five arrays of stride `cap` (label, minx, maxx, miny, maxy); returns the count.
int ref_cc_bounding_box(const int* label, int w, int h, int bgval, int* out, int cap) {
  nscale::ConnComponents cc;
  int count = 0;
  int* box = cc.boundingBox(w, h, label, bgval, count);
  const int m = count < cap ? count : cap;
  for (int f = 0; f < 5; ++f)
    for (int k = 0; k < m; ++k) out[f * cap + k] = box[f * count + k];
  free(box);
  return count;
}

}  // extern "C"
