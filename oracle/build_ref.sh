#!/bin/sh
# TEST INFRASTRUCTURE ONLY.
#
# Builds oracle/_ref/libo3dref_<core>.so from the reference's own pair/panel kernels,
# compiled where they lie (no copy of the reference is written anywhere):
#   src/MathHelper.h  (included through -I)
#   src/CoreFunc.h    (streamed; for RM/EXP/V2 the hard-wired `#define USE_WL_KERNEL`
#                      at CoreFunc.h:37 is switched to the chosen core in the stream,
#                      the switch the reference documents at CoreFunc.h:35-39)
#   src/Kernels.h     (streamed; its `#include "CoreFunc.h"` is dropped because the
#                      switched CoreFunc.h precedes it in the same stream)
#   oracle/ref_driver.cpp (this project's restatement of the loops around them)
# and oracle/_ref/libo3dref_reflect.so from the reference's Reflect.h (streamed without
# its includes of Omega3D.h / Points.h / Surfaces.h, which need Eigen and Vc; the
# declarations it uses come from oracle/reflect_prelude.h) with oracle/ref_reflect_driver.cpp,
# and oracle/_ref/libo3dref_splitmerge.so from the reference's Split.h and Merge.h (each
# streamed up to its *_operation wrapper, which needs the element classes) with the
# vendored lib/nanoflann/nanoflann.hpp, oracle/eigen_shim (a stand-in for the few Eigen
# members they use), oracle/splitmerge_prelude.h and oracle/ref_splitmerge_driver.cpp,
# and oracle/_ref/libo3dref_ovoid.so from the reference's icosahedral sphere:
# src/GeomHelper.cpp streamed up to generate_cuboid (generate_ovoid alone),
# src/IglRefine.cpp, and the vendored lib/igl upsample.cpp,
# triangle_triangle_adjacency.cpp, vertex_triangle_adjacency.cpp and cumsum.cpp, each
# streamed up to its explicit-instantiation block and compiled with IGL_STATIC_LIBRARY
# (so the igl headers do not pull in the rest of igl), against oracle/eigen_shim_igl (a
# stand-in for the Eigen members they use), with oracle/ref_ovoid_driver.cpp,
# and oracle/_ref/libo3dref_vtk.so from the reference's src/VtkXmlWriter.h with the vendored
# lib/tinyxml2 (tinyxml2.cpp compiled) and lib/cppcodec, driven by oracle/ref_vtk_driver.cpp.
#
# The reference is looked for in a checkout named `reference` beside this repository's
# checkout (../reference/src relative to the repository root); set O3D_REFERENCE_SRC to
# its src/ directory to use another location.  When the sources are absent (e.g. on a
# machine without the reference) the script prints a note and exits 0: the ref libraries
# are a checker, not the product.
set -e
HERE="$(cd "$(dirname "$0")" && pwd)"
REF="${O3D_REFERENCE_SRC:-$(dirname "$(dirname "$HERE")")/reference/src}"
OUT="$HERE/_ref"
if [ ! -f "$REF/Kernels.h" ] || [ ! -f "$REF/CoreFunc.h" ] || [ ! -f "$REF/MathHelper.h" ]; then
  echo "build_ref: reference sources not found under $REF; oracle/_ref not built"
  exit 0
fi
CXX="${CXX:-g++}"
mkdir -p "$OUT"
for core in RM WL EXP V2; do
  lc=$(echo "$core" | tr 'A-Z' 'a-z')
  macro="$core"
  [ "$core" = EXP ] && macro=EXPONENTIAL
  {
    if [ "$core" = WL ]; then
      cat "$REF/CoreFunc.h"
    else
      sed -e 's|^#define USE_WL_KERNEL|/* WL switched off for this build */|' \
          -e "s|^//#define USE_${macro}_KERNEL|#define USE_${macro}_KERNEL|" "$REF/CoreFunc.h"
    fi
    sed -e 's|^#include "CoreFunc.h"|/* CoreFunc.h streamed above */|' "$REF/Kernels.h"
    cat "$HERE/ref_driver.cpp"
  } | "$CXX" -std=c++17 -O2 -ffp-contract=off -fopenmp -fPIC -shared -w -I"$REF" -x c++ - \
        -o "$OUT/libo3dref_$lc.so"
  echo "build_ref: built $OUT/libo3dref_$lc.so"
done
if [ -f "$REF/Reflect.h" ]; then
  {
    cat "$HERE/reflect_prelude.h"
    sed -e 's|^#include "Omega3D.h"|/* declared in reflect_prelude.h */|' \
        -e 's|^#include "Points.h"|/* declared in reflect_prelude.h */|' \
        -e 's|^#include "Surfaces.h"|/* declared in reflect_prelude.h */|' "$REF/Reflect.h"
    cat "$HERE/ref_reflect_driver.cpp"
  } | "$CXX" -std=c++17 -O2 -ffp-contract=off -fopenmp -fPIC -shared -w -I"$REF" -x c++ - \
        -o "$OUT/libo3dref_reflect.so"
  echo "build_ref: built $OUT/libo3dref_reflect.so"
fi
NANOFLANN="${O3D_REFERENCE_LIB:-$REF/../lib}"
if [ -f "$REF/Split.h" ] && [ -f "$REF/Merge.h" ] && [ -f "$NANOFLANN/nanoflann/nanoflann.hpp" ]; then
  {
    cat "$HERE/splitmerge_prelude.h"
    sed -n '1,/^\/\/ split any collections of Points/p' "$REF/Split.h"
    sed -n '1,/^\/\/ run some number of merge ops/p' "$REF/Merge.h"
    cat "$HERE/ref_splitmerge_driver.cpp"
  } | "$CXX" -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w -I"$REF" -I"$NANOFLANN" \
        -I"$HERE/eigen_shim" -x c++ - -o "$OUT/libo3dref_splitmerge.so"
  echo "build_ref: built $OUT/libo3dref_splitmerge.so"
fi
IGL="$NANOFLANN/igl"
if [ -f "$REF/GeomHelper.cpp" ] && [ -f "$REF/IglRefine.cpp" ] && [ -f "$IGL/upsample.cpp" ]; then
  {
    printf '#define IGL_STATIC_LIBRARY\n#define IGL_PARALLEL_FOR_FORCE_SERIAL\n'
    for f in cumsum vertex_triangle_adjacency triangle_triangle_adjacency upsample; do
      sed -n '/^#ifdef IGL_STATIC_LIBRARY/q;p' "$IGL/$f.cpp"
    done
    cat "$REF/IglRefine.cpp"
    sed -n '/^ElementPacket<float> generate_cuboid/q;p' "$REF/GeomHelper.cpp"
    cat "$HERE/ref_ovoid_driver.cpp"
  } | "$CXX" -std=c++17 -O2 -ffp-contract=off -fPIC -shared -w -I"$REF" -I"$NANOFLANN" -I"$IGL" \
        -I"$HERE/eigen_shim_igl" -x c++ - -o "$OUT/libo3dref_ovoid.so"
  echo "build_ref: built $OUT/libo3dref_ovoid.so"
fi
if [ -f "$REF/VtkXmlWriter.h" ] && [ -f "$NANOFLANN/tinyxml2/tinyxml2.cpp" ] && [ -d "$NANOFLANN/cppcodec" ]; then
  "$CXX" -std=c++17 -O2 -fPIC -shared -w -I"$REF" -I"$NANOFLANN" "$NANOFLANN/tinyxml2/tinyxml2.cpp" \
        "$HERE/ref_vtk_driver.cpp" -o "$OUT/libo3dref_vtk.so"
  echo "build_ref: built $OUT/libo3dref_vtk.so"
fi
