#!/bin/sh
# Builds the oracle pin: PhiNum's own hot-path sources, compiled unchanged
# from the reference tree (REF_DIR, default /root/reference) against the
# single-rank MPI/FFTW shims in oracle/ref_shim/, into oracle/_ref/.
#
# Test infrastructure only.  Flags: no -ffast-math and no FP contraction, so
# that the reference's FP64 arithmetic is plain IEEE round-to-nearest in
# source order (the reference's own PBS scripts add -ffast-math, which lets
# the compiler reorder; the parity pin wants the source order).  Exits 0
# without building when the reference tree is absent.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF_DIR="${REF_DIR:-/root/reference}"
OUT="$HERE/_ref"
if [ ! -f "$REF_DIR/dynamics.cpp" ]; then
  echo "build_ref: reference tree not found at $REF_DIR; skipping"
  exit 0
fi
mkdir -p "$OUT"
CXXFLAGS="-std=gnu++14 -O2 -ffp-contract=off -fno-fast-math -fPIC -shared"
build() {
  name="$1"; shift
  g++ $CXXFLAGS "$@" -I"$HERE/ref_shim" -I"$REF_DIR" "$HERE/ref_driver.cpp" -o "$OUT/$name"
}
build libphinum_ref_t0_f64.so -DPHN_REF_THEORY=0 -DPHN_REF_PRECISION=0 &
build libphinum_ref_t1_f64.so -DPHN_REF_THEORY=1 -DPHN_REF_PRECISION=0 &
build libphinum_ref_t0_f32.so -DPHN_REF_THEORY=0 -DPHN_REF_PRECISION=-1 &
build libphinum_ref_t1_f32.so -DPHN_REF_THEORY=1 -DPHN_REF_PRECISION=-1 &
for t in 2 3 4 5; do
  build libphinum_ref_t${t}_f64.so -DPHN_REF_THEORY=$t -DPHN_REF_PRECISION=0 &
done
wait
# the other initial conditions: initialize 0, 1, 2, 4, and the charged
# variant (withcharge 1) of initialize 2 and 3
for i in 0 1 2 4; do
  build libphinum_ref_t0_f64_ic${i}.so -DPHN_REF_THEORY=0 -DPHN_REF_PRECISION=0 -DPHN_REF_INIT=$i &
done
for i in 2 3; do
  build libphinum_ref_t0_f64_ic${i}q.so -DPHN_REF_THEORY=0 -DPHN_REF_PRECISION=0 -DPHN_REF_INIT=$i \
    -DPHN_REF_WITHCHARGE=1 &
done
wait
# the energy-density analysis (withEnergyPS 1, EnergybasedID 1): the
# theories for which the reference compiles it (its theory 0 and 1 forms
# name the monodromy mass, which only theory 3 defines)
for t in 2 3 4 5; do
  build libphinum_ref_t${t}_f64_eps.so -DPHN_REF_THEORY=$t -DPHN_REF_PRECISION=0 -DPHN_REF_ENERGYPS=1 \
    -DPHN_REF_ENERGYID=1 &
done
build libphinum_ref_t3_f64_exp_eps.so -DPHN_REF_THEORY=3 -DPHN_REF_PRECISION=0 -DPHN_REF_EXPANSION=1 \
  -DPHN_REF_ENERGYPS=1 -DPHN_REF_ENERGYID=1 &
wait
# the expanding box (expansion 1), every theory
for t in 0 1 2 3 4 5; do
  build libphinum_ref_t${t}_f64_exp.so -DPHN_REF_THEORY=$t -DPHN_REF_PRECISION=0 -DPHN_REF_EXPANSION=1 &
done
wait
ls -1 "$OUT"
