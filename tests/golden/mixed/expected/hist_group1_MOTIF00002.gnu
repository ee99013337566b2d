set output "hist_group1_MOTIF00002.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-71.33:23.3206]
set yrange [0:166051]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00002.dat" using 1:2 title 'MOTIF00002 (group1)' with boxes
