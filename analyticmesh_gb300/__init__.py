"""GB300-native Analytic Marching."""
