"""GB300-native kinetic step of the RREA overlay (e-/e+/photon transport)."""
import os

PACKAGE_DIR = os.path.dirname(os.path.abspath(__file__))
REPO_ROOT = os.path.dirname(PACKAGE_DIR)
DEFAULT_TABLES = os.path.join(REPO_ROOT, "data", "schema6", "transport_physics.json")
# the dry-air electron closure of the carrier fluid's table models
DEFAULT_CLOSURE = os.path.join(REPO_ROOT, "data", "closure", "dry_air_swarm_hybrid_v3.csv")
