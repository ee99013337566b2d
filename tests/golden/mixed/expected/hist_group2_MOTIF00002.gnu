set output "hist_group2_MOTIF00002.ps"
set key autotitle columnhead
set terminal postscript landscape
set terminal postscript noenhanced
set xrange [-71.4643:22.6781]
set yrange [0:168832]
set xlabel 'PWM score'
set ylabel 'count'
plot "hist_group2_MOTIF00002.dat" using 1:2 title 'MOTIF00002 (group2)' with boxes
