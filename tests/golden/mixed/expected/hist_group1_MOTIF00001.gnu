set output "hist_group1_MOTIF00001.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-47.2175:11.6076]
set yrange [0:128805]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group1_MOTIF00001.dat" using 1:2 title 'MOTIF00001 (group1)' with boxes
