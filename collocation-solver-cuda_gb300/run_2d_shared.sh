#!/bin/bash
# Drop-in for the reference's run_2d_shared.sh: ./run_2d_shared.sh <ocp> [m]
arg_m=${2:-4}
exec python "$(dirname "$0")/cli.py" "$1" -m "$arg_m"
