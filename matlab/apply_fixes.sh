#!/bin/sh
# apply_fixes.sh -- the one MATLAB-class fix FrameLab needs to run its fan-beam
# adjoint through this library, applied to the user's own FrameLab checkout
# (the reference's files are not shipped here).
#
#   sh matlab/apply_fixes.sh /path/to/FrameLab
#
# +Operators/@FanBeamScanner/applyAdjoint.m compares the scanner's para with
# object.para, a field the object does not have; the cone scanner's
# applyAdjoint.m reads object.scanner.para. The fan scanner is given the same
# read. The edit is idempotent: a checkout already fixed is left as it is.
set -eu
root=${1:?usage: apply_fixes.sh /path/to/FrameLab}
f="$root/matlab/classes/+Operators/@FanBeamScanner/applyAdjoint.m"
[ -f "$f" ] || { echo "not found: $f" >&2; exit 1; }
sed -i 's/structcmp(this\.para,object\.para)/structcmp(this.para,object.scanner.para)/; s/this\.para = object\.para;/this.para = object.scanner.para;/' "$f"
grep -q 'object\.scanner\.para' "$f" && echo "fixed: $f"
