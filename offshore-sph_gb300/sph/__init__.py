"""GB300-native WCSPH step behind Offshore-SPH's plugin surface."""
