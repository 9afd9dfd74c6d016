"""GB300-native implementation of the SW2 shallow-water step."""
