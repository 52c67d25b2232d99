"""GB300-native WABBIT ACM block-level time-step hot path."""
