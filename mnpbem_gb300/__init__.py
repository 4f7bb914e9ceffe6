"""GB300-native retarded BEM hot path of MNPBEM (compgreenret + bemret + planewave spectra)."""
