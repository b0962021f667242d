"""GB300-native LightFEM solve path (package root; filled in below)."""
