#!/bin/sh
# Oracle build recipe (test infrastructure only): where the unmodified reference tree is.
#
#   sh oracle/reference_tree.sh        prints the directory holding Box2DRef/ (the reference's
#                                      Regression/box2d-ref tree), or nothing when it is absent.
#
# B2_REFERENCE_TREE overrides the location; the fallback is where this build's container mounts
# the reference (read-only). The GPU host has no reference tree: there the script prints nothing
# and the oracle uses only the CPU restatement and the committed golden vectors.
REF="${B2_REFERENCE_TREE:-/root/reference/Regression/box2d-ref}"
if [ -d "$REF/Box2DRef" ]; then
    echo "$REF"
fi
