#!/bin/sh
# Writes the two configuration headers that the reference's sources include
# (esl_config.h, p7_config.h) into OUTDIR, by switching on the few settings
# an x86-64 Linux/glibc build with SSE2 needs in the reference's own .in
# templates. This replaces running the reference's autoconf script: only
# the defines listed below are set, everything else stays #undef.
#   usage: mkconfig.sh REFCODE OUTDIR
set -e
REF="$1"; OUT="$2"
mkdir -p "$OUT"
on() { printf 's|^#undef %s\\b.*$|#define %s %s|\n' "$1" "$1" "$2"; }
{
  on EASEL_VERSION '"h3.1b1"'
  on EASEL_DATE '"May 2013"'
  on EASEL_COPYRIGHT '"(c) HHMI"'
  on EASEL_LICENSE '"GPLv3"'
  on eslDEBUGLEVEL 0
  on eslLIBRARY 1
  for h in HAVE_INTTYPES_H HAVE_STDINT_H HAVE_UNISTD_H HAVE_SYS_TYPES_H \
           HAVE_STRINGS_H HAVE_EMMINTRIN_H HAVE_PMMINTRIN_H HAVE_XMMINTRIN_H \
           HAVE_SSE2 HAVE_SSE2_CAST HAVE_CHMOD HAVE_FSEEKO HAVE_FSTAT HAVE_GETCWD \
           HAVE_GETPID HAVE_MKSTEMP HAVE_POPEN HAVE_PUTENV HAVE_STAT \
           HAVE_STRCASECMP HAVE_SYSCONF HAVE_TIMES; do on "$h" 1; done
} > "$OUT/esl.sed"
{
  on HMMER_VERSION '"3.1b1"'
  on HMMER_DATE '"May 2013"'
  on HMMER_COPYRIGHT '"(c) HHMI"'
  on HMMER_LICENSE '"GPLv3"'
  on HMMER_URL '"http://hmmer.org/"'
  on p7_IMPL_SSE 1
  on HAVE_SSE2 1
} > "$OUT/p7.sed"
sed -f "$OUT/esl.sed" "$REF/easel/esl_config.h.in" > "$OUT/esl_config.h"
sed -f "$OUT/p7.sed"  "$REF/src/p7_config.h.in"  > "$OUT/p7_config.h"
