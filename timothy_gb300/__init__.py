"""GB300-native Timothy cell-mechanics hot path."""
