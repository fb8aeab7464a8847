"""GB300-native CRTM forward / K-matrix / adjoint path (ODPS + Emission/ADA/SOI)."""
