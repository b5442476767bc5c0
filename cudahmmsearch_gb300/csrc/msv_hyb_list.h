// msv_hyb_list.h -- the (DP words per lane, lanes, 8-bit words) triples for
// which the mixed-width lane-group SSV kernel is compiled (inst_hyb*.cu) and
// dispatched (msv_api.cu): the default share of every width (msvgb_detail::
// hyb_default_words, 32-lane groups included) and two wider ones.
#pragma once
#define MSVGB_HYB_LIST(X) \
  X(10, 8, 4) X(11, 8, 4) X(12, 8, 4) X(13, 8, 4) \
  X(14, 8, 4) X(15, 8, 4) X(16, 8, 4) X(17, 8, 4) \
  X(18, 8, 8) X(19, 8, 8) X(20, 8, 8) X(21, 8, 8) \
  X(22, 8, 8) X(23, 8, 8) X(24, 8, 8) X(25, 8, 8) \
  X(26, 8, 8) X(27, 8, 8) X(28, 8, 8) X(29, 8, 8) \
  X(30, 8, 8) X(31, 8, 8) X(32, 8, 8) X(13, 16, 4) \
  X(14, 16, 4) X(15, 16, 4) X(16, 16, 4) X(17, 16, 4) \
  X(18, 16, 4) X(19, 16, 4) X(20, 16, 4) X(21, 16, 4) \
  X(22, 16, 4) X(23, 16, 4) X(24, 16, 8) X(25, 16, 8) \
  X(26, 16, 8) X(27, 16, 8) X(28, 16, 8) X(29, 16, 8) \
  X(30, 16, 8) X(31, 16, 8) X(32, 16, 8) X(26, 8, 12) \
  X(32, 8, 16) \
  X(17, 32, 8) X(18, 32, 8) X(19, 32, 8) X(20, 32, 8) X(21, 32, 8) X(22, 32, 8) X(23, 32, 8) X(24, 32, 8) \
  X(25, 32, 8) X(26, 32, 8) X(27, 32, 8) X(28, 32, 8) X(29, 32, 8) X(30, 32, 8) X(31, 32, 8) X(32, 32, 8) \

