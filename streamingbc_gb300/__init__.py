"""GB300-native StreamingBC hot path."""
