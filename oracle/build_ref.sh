#!/bin/sh
# Build the unmodified reference skid (N-BodyShop/skid v1.4.1) from its own
# source files, where they lie, into oracle/_ref/.  Test infrastructure only:
# the binaries are the oracle's reference leg and never part of the product.
#
#   oracle/_ref/skid       reference skid, as shipped
#   oracle/_ref/skid_nsp   patched oracle for -nsp (every scatterer kept; see
#                          oracle/nsp_shim.c), built without editing or
#                          copying a reference source file
#
# The only missing dependency is SunRPC/tirpc XDR; oracle/xdr_shim provides
# the handful of XDR routines the reference calls.  -ffp-contract=off keeps
# a*b+c unfused on hosts whose gcc contracts to FMA by default (aarch64).
#
# Usage: sh oracle/build_ref.sh <reference-source-dir>
#   (or SKID_REF_DIR=<dir> sh oracle/build_ref.sh); oracle.py passes the
#   staged copy baseline/_ref/src.
set -eu
REF=${1:-${SKID_REF_DIR:-}}
if [ -z "$REF" ]; then
    echo "build_ref: give the reference source directory (argument or SKID_REF_DIR)" >&2
    exit 2
fi
HERE=$(cd "$(dirname "$0")" && pwd)
OUT="$HERE/_ref"
if [ ! -f "$REF/kd.c" ]; then
    echo "build_ref: no reference sources at $REF" >&2
    exit 2
fi
mkdir -p "$OUT"
CFLAGS="-O2 -ffp-contract=off -D_GNU_SOURCE -w -I$HERE/xdr_shim"
gcc $CFLAGS -o "$OUT/skid" \
    "$REF/main.c" "$REF/kd.c" "$REF/smooth1.c" "$REF/grav.c" \
    "$REF/cosmo.c" "$REF/romberg.c" "$REF/runge.c" \
    "$HERE/xdr_shim/xdr_shim.c" -lm
echo "build_ref: built $OUT/skid"
# -nsp oracle: smooth1.c as a shared object (-fPIC leaves its global
# functions interposable, so its call to ScatterCut goes through the PLT);
# the executable exports its own ScatterCut from nsp_shim.c (-rdynamic) and
# the dynamic linker binds the call there.  main.c alone is compiled with
# bAllowInitialCut renamed to the shim's nsp_no_initial_cut.
TMPO=$(mktemp -d)
trap 'rm -rf "$TMPO"' EXIT
gcc $CFLAGS -fPIC -fno-inline -shared -o "$OUT/libsmooth1_nsp.so" "$REF/smooth1.c"
gcc $CFLAGS -DbAllowInitialCut=nsp_no_initial_cut -c -o "$TMPO/main_nsp.o" "$REF/main.c"
gcc $CFLAGS -rdynamic -o "$OUT/skid_nsp" "$TMPO/main_nsp.o" \
    "$REF/kd.c" "$REF/grav.c" "$REF/cosmo.c" "$REF/romberg.c" "$REF/runge.c" \
    "$HERE/xdr_shim/xdr_shim.c" "$HERE/nsp_shim.c" \
    -L"$OUT" -lsmooth1_nsp -Wl,-rpath,'$ORIGIN' -lm
echo "build_ref: built $OUT/skid_nsp"
