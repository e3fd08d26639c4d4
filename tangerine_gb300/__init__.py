"""GB300-native (sm_103a) CSG signed-distance evaluation and export meshing for Tangerine."""
