"""adeco_gb300 -- GB300-native phase-space tetrahedron mass deposit."""
