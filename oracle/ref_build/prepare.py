#!/usr/bin/env python3
"""Stage the reference's own C++ sources for the CPU oracle / CPU baseline build.

TEST INFRASTRUCTURE ONLY.  Nothing in the product (``vortegrid_gb300``) imports,
links or executes anything that this script produces.

What it does:
  1. copies the reference translation units that the VortonSim step needs from
     ``<reference>/Samples/MjgIntelFluidDemo_Part20`` into ``oracle/_ref/src``
     (git-ignored; the copy travels to the GPU host with the working tree so
     that ``oracle/ref_build/Makefile`` can rebuild it there for that CPU);
  2. applies the minimal set of LP64/GCC portability edits the MSVC-era code
     needs (each edit is listed below with the reason).  No arithmetic is
     changed: every edit is a type fix, a missing ``template<>``, or a
     replacement of a type-punning cast by ``memcpy`` with identical bits.

The reference sources are never committed; only this recipe is.
"""
import os
import re
import shutil
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE = os.path.dirname(HERE)
SAMPLE = os.path.join("Samples", "MjgIntelFluidDemo_Part20")
DST = os.path.join(ORACLE, "_ref", "src")

SUBDIRS = ["Core", "VortonFluid", "Particles", "Sim", "FluidBodySim",
           "SmoothedPclHydro", "Impulsion", "Collision"]

# (relative file, regex, replacement, reason).  Each regex must match exactly
# the stated number of times or the script fails loudly.
EDITS = [
    # LP64: GetNumPoints() returns `const unsigned &`; with size_t storage it
    # binds to a temporary (dangling reference).  32-bit MSVC had both 4 bytes.
    ("Core/SpatialPartition/uniformGrid.h",
     r"size_t(\s+)mNumPoints\[ 3 \] ;", r"unsigned\1mNumPoints[ 3 ] ;", 1,
     "LP64: point counts stored as 32-bit like the original 32-bit build"),
    # GCC rejects calling a member template of an incomplete NestedGrid<T>
    # from inside UniformGrid; route through an equivalent free function.
    ("Core/SpatialPartition/uniformGrid.h",
     r"NestedGrid<ItemT>::GetChildClusterMinCornerIndex\(",
     "VgRefChildClusterMinCornerIndex(", 2,
     "GCC two-phase lookup: NestedGrid is incomplete where UniformGrid uses it"),
    # mat33.h: `static friend` is an MSVC extension.
    ("Core/Math/mat33.h", r"static friend Vec3 operator\*", "friend Vec3 operator*", 1,
     "GCC: static friend is ill-formed"),
    # math.h: `(long&) float` reads 8 bytes on LP64.  memcpy of 4 bytes keeps
    # the exact IEEE bit pattern the 32-bit original used.
    ("Core/Math/math.h", r"long    i   = \(long&\) val ;",
     "int32_t i ; memcpy( &i , &val , 4 ) ;", 3,
     "LP64: long is 8 bytes; the magic-constant rsqrt needs a 32-bit pun"),
    ("Core/Math/math.h", r"float   y   = \(float&\) i ;",
     "float y ; memcpy( &y , &i , 4 ) ;", 2, "LP64: matching 32-bit pun back"),
    ("Core/Math/math.h", r"    y   = \(float&\) i ;",
     "    memcpy( &y , &i , 4 ) ;", 1, "LP64: macro variant of the pun"),
    # Explicit specialisations need template<> in standard C++.
    ("Core/SpatialPartition/uniformGridMath.cpp",
     r"\nvoid UniformGrid<Mat33>::ComputeStatistics", "\ntemplate<> void UniformGrid<Mat33>::ComputeStatistics", 1,
     "C++ standard: explicit specialisation"),
    ("Particles/particleDiagnostics.cpp",
     r"\nvoid UniformGrid<Particle>::GenerateBrickOfBytes", "\ntemplate<> void UniformGrid<Particle>::GenerateBrickOfBytes", 1,
     "C++ standard: explicit specialisation"),
    # Declaration in vortonSim.h uses size_t; definition used unsigned.
    ("VortonFluid/vortonSim.cpp",
     r"ComputeVelocityAtVortons_Slice\( unsigned iPclStart , unsigned iPclEnd ,",
     "ComputeVelocityAtVortons_Slice( size_t iPclStart , size_t iPclEnd ,", 1,
     "definition must match the size_t declaration in vortonSim.h"),
    ("VortonFluid/vortonSim.cpp", r"static const sBoundariesOnly = true ;",
     "static const bool sBoundariesOnly = true ;", 1, "implicit int is ill-formed C++"),
    ("FluidBodySim/fluidBodySim.cpp", r"size_t(\s+)idxPlane ;", r"unsigned\1idxPlane ;", 1,
     "LP64: passed where unsigned& is expected"),
]


def copy_tree(ref):
    if os.path.isdir(DST):
        shutil.rmtree(DST)
    for sub in SUBDIRS:
        for root, _dirs, files in os.walk(os.path.join(ref, sub)):
            for f in files:
                if not f.endswith((".h", ".cpp", ".inl")):
                    continue
                src = os.path.join(root, f)
                rel = os.path.relpath(src, ref)
                out = os.path.join(DST, rel)
                os.makedirs(os.path.dirname(out), exist_ok=True)
                shutil.copyfile(src, out)
    # Case-sensitive include used by SmoothedPclHydro ("Core/Math/Vec2.h").
    v2 = os.path.join(DST, "Core", "Math", "vec2.h")
    if os.path.exists(v2):
        shutil.copyfile(v2, os.path.join(DST, "Core", "Math", "Vec2.h"))


def apply_edits():
    for rel, pat, rep, count, why in EDITS:
        if rep is None:
            continue
        path = os.path.join(DST, rel)
        with open(path, "r", encoding="latin-1") as fh:
            text = fh.read()
        new, n = re.subn(pat, rep, text)
        if n != count:
            sys.exit(f"prepare.py: edit '{why}' matched {n}x in {rel}, expected {count}")
        with open(path, "w", encoding="latin-1") as fh:
            fh.write(new)
    # uniformGrid.h: add the free function used above, plus two index-type
    # overloads GCC needs for LP64 (same arithmetic as the existing members).
    path = os.path.join(DST, "Core/SpatialPartition/uniformGrid.h")
    with open(path, "r", encoding="latin-1") as fh:
        text = fh.read()
    anchor = "template <class ItemT> class UniformGrid : public UniformGridGeometry"
    assert text.count(anchor) == 1, "uniformGrid.h anchor"
    helper = ("inline void VgRefChildClusterMinCornerIndex( unsigned c[3] , const unsigned d[3] , const unsigned p[3] )"
              " { c[0] = p[0] * d[0] ; c[1] = p[1] * d[1] ; c[2] = p[2] * d[2] ; }\n\n")
    text = text.replace(anchor, helper + anchor)
    anchor2 = "    protected:\n\n        /** Precompute grid spacing"
    assert text.count(anchor2) == 1, "uniformGrid.h anchor2"
    overloads = (
        "        size_t OffsetFromIndices( const unsigned indices[3] ) const\n"
        "        { return OffsetFromIndices( size_t( indices[0] ) , size_t( indices[1] ) , size_t( indices[2] ) ) ; }\n"
        "        void PositionFromIndices( Vec3 & vPosition , const size_t indices[3] ) const\n"
        "        { const unsigned u[3] = { unsigned( indices[0] ) , unsigned( indices[1] ) , unsigned( indices[2] ) } ; PositionFromIndices( vPosition , u ) ; }\n\n")
    text = text.replace(anchor2, overloads + anchor2)
    # RemoveComponent uses a size_t[4] index buffer with an unsigned[4] API.
    text, n = re.subn(r"size_t(\s+)indices\[4\] ; // Indices of grid cell containing position\.",
                      r"unsigned\1indices[4] ; // Indices of grid cell containing position.", text)
    with open(path, "w", encoding="latin-1") as fh:
        fh.write(text)
    for rel in ("Core/SpatialPartition/nestedGridDiagnostics.cpp",):
        p = os.path.join(DST, rel)
        if os.path.exists(p):
            with open(p, "r", encoding="latin-1") as fh:
                t = fh.read()
            t = re.sub(r"\n/\* static \*/ void NestedGrid<", "\ntemplate<> /* static */ void NestedGrid<", t)
            with open(p, "w", encoding="latin-1") as fh:
                fh.write(t)


def reference_sample(root):
    """The newest sample snapshot inside a VorteGrid checkout at `root` (or
    `root` itself when it already is that snapshot)."""
    inner = os.path.join(root, SAMPLE)
    return inner if os.path.isdir(inner) else root


def main():
    # The checkout's location comes from the command line or VG_REFERENCE_TREE;
    # there is no built-in default.
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("VG_REFERENCE_TREE", "")
    if not root:
        print("prepare.py: give the VorteGrid checkout as an argument or in VG_REFERENCE_TREE; nothing staged")
        return 1
    ref = reference_sample(root)
    if not os.path.isdir(ref):
        print(f"prepare.py: reference tree not found at {ref}; nothing staged")
        return 1
    copy_tree(ref)
    apply_edits()
    with open(os.path.join(DST, ".staged"), "w") as fh:
        fh.write(ref + "\n")
    print(f"prepare.py: staged reference sources into {DST}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
