"""Script-facing names of bricklib's stencil language (codegen/st), re-implemented so the
reference's stencil scripts run unchanged and lower to tap lists (bricklib_gb300.dsl)."""
