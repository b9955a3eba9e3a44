#!/usr/bin/env bash
# Compile the reference's own RHS-path sources (unmodified, where they lie)
# into oracle/_ref/ against the AMReX stand-in in oracle/ref_shim/.
# Test infrastructure only: the outputs are oracles, never product code.
#
#   bash oracle/build_ref.sh REFERENCE_ROOT     (or AMRS_REFERENCE_ROOT set)
#
# Two libraries, one per closure family the reference ships
# (src/cls/Closures.h): constant viscosity/conductivity and Sutherland.
set -euo pipefail
REF="${1:-${AMRS_REFERENCE_ROOT:?usage: build_ref.sh REFERENCE_ROOT (or set AMRS_REFERENCE_ROOT)}}"
HERE="$(cd "$(dirname "$0")" && pwd)"
OUT="$HERE/_ref"
mkdir -p "$OUT"
INC=(-I"$HERE/ref_shim" -I"$REF/src" -I"$REF/src/rhs" -I"$REF/src/cls" -I"$REF/src/tim")
FLAGS=(-std=c++20 -O2 -ffp-contract=off -fPIC -shared -w)
build() {
  local name="$1"; shift
  g++ "${FLAGS[@]}" "${INC[@]}" "$@" -o "$OUT/$name.tmp" \
      "$REF/src/tim/CNS_advance.cpp" "$HERE/ref_driver.cpp"
  mv "$OUT/$name.tmp" "$OUT/$name"
}
build libcnsref_const.so -DREF_VISC=visc_const_t -DREF_COND=cond_const_t -DREF_CONST_TRANSPORT=1 &
build libcnsref_suth.so -DREF_VISC=visc_suth_t -DREF_COND=cond_suth_t &
wait
echo "$OUT"
