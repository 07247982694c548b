#!/bin/bash
# pipeline.sh <flow_case> <velocity_set> <id> [pflbm_run options]
# Drop-in for the reference's pipeline.sh: clean bin/<case>/<set>/<id>,
# build, run. Output goes to bin/<case>/<set>/<id>/ with the reference's
# file layout. Extra arguments are passed to the driver (see pflbm_run).
set -euo pipefail
GPU_INDEX=${GPU_INDEX:-0}
FLOW_CASE=${1:-}
VELOCITY_SET=${2:-}
ID=${3:-}
if [ -z "$FLOW_CASE" ] || [ -z "$VELOCITY_SET" ] || [ -z "$ID" ]; then
    echo "Error: Insufficient arguments."
    echo "Usage: ./pipeline.sh <flow_case> <velocity_set> <id>"
    echo "Example: ./pipeline.sh JET D3Q19 000"
    exit 1
fi
case "$FLOW_CASE" in JET|DROPLET) ;; *) echo "Invalid flow_case. Use 'JET' or 'DROPLET'."; exit 1 ;; esac
case "$VELOCITY_SET" in D3Q19|D3Q27) ;; *) echo "Invalid velocity_set. Use 'D3Q19' or 'D3Q27'."; exit 1 ;; esac
# the id names a directory that is emptied below: letters, digits, '_' and '-' only
if ! [[ "$ID" =~ ^[A-Za-z0-9_-]+$ ]]; then
    echo "Invalid id '$ID': use letters, digits, '_' or '-'."
    exit 1
fi
shift 3
BASE_DIR="$(cd -- "$(dirname -- "${BASH_SOURCE[0]}")" &>/dev/null && pwd)"
SIMULATION_DIR="${BASE_DIR}/bin/${FLOW_CASE}/${VELOCITY_SET}/${ID}"
mkdir -p "${SIMULATION_DIR}"
find "${SIMULATION_DIR}" -mindepth 1 ! -name ".gitkeep" -exec rm -rf {} +
cd "${BASE_DIR}"
GPU_ARCH=103 bash "${BASE_DIR}/compile.sh" "${FLOW_CASE}" "${VELOCITY_SET}" "${ID}"
EXECUTABLE="${BASE_DIR}/bin/${FLOW_CASE}/${VELOCITY_SET}/${ID}sim_${FLOW_CASE}_${VELOCITY_SET}_sm103"
export GPU_INDEX
"${EXECUTABLE}" "${FLOW_CASE}" "${VELOCITY_SET}" "${ID}" 1 "$@"
echo "Process completed successfully!"
