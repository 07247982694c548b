#!/bin/bash
# compile.sh <FLOW_CASE> <VELOCITY_SET> <ID>
# Same interface as the reference's compile.sh. The GB300 library is
# configured at run time, so this builds libpflbm.so and the pflbm_run driver
# once (sm_103a) and places the driver at the executable path the reference
# uses: bin/<case>/<set>/<id>sim_<case>_<set>_sm<CC>.
set -euo pipefail
FLOW_CASE=${1:-}
VELOCITY_SET=${2:-}
ID=${3:-}
if [ -z "$FLOW_CASE" ] || [ -z "$VELOCITY_SET" ] || [ -z "$ID" ]; then
    echo "Usage: ./compile.sh <FLOW_CASE> <VELOCITY_SET> <ID>"
    echo "Example: ./compile.sh JET D3Q19 000"
    exit 1
fi
if [ "$VELOCITY_SET" != "D3Q19" ] && [ "$VELOCITY_SET" != "D3Q27" ]; then
    echo "Invalid VELOCITY_SET. Use 'D3Q19' or 'D3Q27'."
    exit 1
fi
if ! [[ "$ID" =~ ^[A-Za-z0-9_-]+$ ]]; then
    echo "Invalid ID '$ID': use letters, digits, '_' or '-'."
    exit 1
fi
BASE_DIR="$(cd -- "$(dirname -- "${BASH_SOURCE[0]}")" &>/dev/null && pwd)"
CC=${GPU_ARCH:-103}
OUTPUT_DIR="${BASE_DIR}/bin/${FLOW_CASE}/${VELOCITY_SET}"
EXECUTABLE="${OUTPUT_DIR}/${ID}sim_${FLOW_CASE}_${VELOCITY_SET}_sm${CC}"
mkdir -p "${OUTPUT_DIR}"
echo "Compiling to ${EXECUTABLE}..."
(cd "${BASE_DIR}" && python3 -c "from phasefieldlbm_gb300 import build; build.build()")
ln -sf "${BASE_DIR}/phasefieldlbm_gb300/_build/pflbm_run" "${EXECUTABLE}"
echo "Compilation completed successfully: ${EXECUTABLE}"
